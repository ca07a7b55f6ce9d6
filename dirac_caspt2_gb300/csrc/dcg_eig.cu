// Hermitian eigensolver on the device (FP64), the replacement of the reference's ZHEEV /
// DSYEV calls (src/diag.F90:43,109).  Eigenvalues come out ascending, as there.
//
// Three phases, each written from the published algorithm:
//   1. Householder reduction of the Hermitian matrix to a real symmetric tridiagonal
//      (Golub & Van Loan, Matrix Computations, 4th ed., 8.3.1) with the complex reflector
//      of LAPACK's documented xLARFG definition (beta real).
//   2. Cuppen's divide and conquer on the tridiagonal (GVL 8.4.4): the tridiagonal is torn
//      into 1x1 leaves by rank-one modifications; sibling blocks are merged level by level.
//      Each merge deflates (small rank-one components, and Givens rotations for pairs of
//      close poles: Dongarra & Sorensen, SIAM J. Sci. Stat. Comput. 8 (1987) s139), solves
//      the secular equation one root per warp with a bracketed two-pole rational model
//      (Bunch, Nielsen & Sorensen, Numer. Math. 31 (1978) 31), recomputes the rank-one
//      vector from the roots so the eigenvectors stay orthogonal (Gu & Eisenstat, SIAM J.
//      Matrix Anal. Appl. 16 (1995) 172), and applies the merge's eigenvector matrix with one
//      batched GEMM per level.
//   3. Back-transformation of the requested eigenvectors by the stored reflectors.
//
// The merge tree is the power-of-two tree: at level l a node covers columns
// [i 2^l, min((i+1) 2^l, n)) and is split after its first 2^(l-1) columns, so a node's
// geometry follows from (l, i) and no tree is stored.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>

#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>

#include "dcg_common.cuh"

namespace dcg {

constexpr double kUnitRoundoff = 1.1102230246251565e-16;   // 2^-53
constexpr int kSecularMaxIter = 100;

__device__ __forceinline__ double eig_warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return __shfl_sync(0xffffffffu, v, 0);   // lane 0's value in every lane
}
__device__ __forceinline__ double eig_warp_prod(double v) {
    for (int o = 16; o > 0; o >>= 1) v *= __shfl_down_sync(0xffffffffu, v, o);
    return __shfl_sync(0xffffffffu, v, 0);
}
__device__ __forceinline__ double eig_warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return __shfl_sync(0xffffffffu, v, 0);
}

// Deterministic block sum (fixed tree); every thread gets the result.  sh >= 32 doubles.
__device__ double eig_block_sum(double v, double *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = eig_warp_sum(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double t = 0.0;
    if (wid == 0) {
        t = lane < nw ? sh[lane] : 0.0;
        t = eig_warp_sum(t);
        if (lane == 0) sh[0] = t;
    }
    __syncthreads();
    t = sh[0];
    __syncthreads();
    return t;
}

__device__ double eig_block_max(double v, double *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    v = eig_warp_max(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double t = 0.0;
    if (wid == 0) {
        t = lane < nw ? sh[lane] : 0.0;
        t = eig_warp_max(t);
        if (lane == 0) sh[0] = t;
    }
    __syncthreads();
    t = sh[0];
    __syncthreads();
    return t;
}

// ===================================================================== 1. tridiagonal reduction
// Step k: reflector for column k (rows k+1..n-1), v stored in A(k+1:n-1, k) with v0 = 1.
__global__ void hh_gen_kernel(int n, int k, cplx *A, int64_t lda, double *d, double *e, cplx *tau) {
    __shared__ double sh[32];
    __shared__ cplx s_scale;
    __shared__ int s_skip;
    const int m = n - k - 1;
    cplx *x = A + (k + 1) + (int64_t)k * lda;
    double s = 0.0;
    for (int i = 1 + threadIdx.x; i < m; i += blockDim.x) s += cabs2(x[i]);
    s = eig_block_sum(s, sh);
    if (threadIdx.x == 0) {
        cplx alpha = x[0];
        double xnorm = sqrt(s);
        cplx t;
        double beta;
        if (xnorm == 0.0 && alpha.y == 0.0) {
            t = mk(0.0, 0.0);
            beta = alpha.x;
            s_skip = 1;
        } else {
            double nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm * xnorm);
            beta = alpha.x >= 0.0 ? -nrm : nrm;
            t = mk((beta - alpha.x) / beta, -alpha.y / beta);
            s_scale = cdiv(mk(1.0, 0.0), mk(alpha.x - beta, alpha.y));
            s_skip = 0;
        }
        tau[k] = t;
        e[k] = beta;
        d[k] = A[k + (int64_t)k * lda].x;
    }
    __syncthreads();
    if (!s_skip)
        for (int i = 1 + threadIdx.x; i < m; i += blockDim.x) x[i] = cmul(x[i], s_scale);
    __syncthreads();
    if (threadIdx.x == 0) x[0] = mk(1.0, 0.0);
}

// partial p(i) = sum_{j in chunk} A(k+1+i, k+1+j) v(j)
constexpr int HH_CHUNK = 256;
__global__ void hh_matvec_kernel(int n, int k, const cplx *__restrict__ A, int64_t lda, const cplx *__restrict__ tau,
                                 cplx *ppart) {
    __shared__ cplx vs[HH_CHUNK];
    const int m = n - k - 1;
    const cplx t = tau[k];
    const int j0 = blockIdx.y * HH_CHUNK;
    const int j1 = min(m, j0 + HH_CHUNK);
    const cplx *v = A + (k + 1) + (int64_t)k * lda;
    for (int j = threadIdx.x; j < j1 - j0; j += blockDim.x) vs[j] = v[j0 + j];
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    cplx acc = mk(0.0, 0.0);
    if (t.x != 0.0 || t.y != 0.0) {
        const cplx *Ai = A + (k + 1 + i) + (int64_t)(k + 1) * lda;
        for (int j = j0; j < j1; j++) cfma(acc, Ai[(int64_t)j * lda], vs[j - j0]);
    }
    ppart[(int64_t)blockIdx.y * n + i] = acc;
}

// w = tau*p + alpha v,  alpha = -1/2 tau (x^H v) with x = tau*p
__global__ void hh_w_kernel(int n, int k, const cplx *A, int64_t lda, const cplx *tau, const cplx *ppart,
                            int nchunk, cplx *w) {
    __shared__ double sh[32];
    const int m = n - k - 1;
    const cplx t = tau[k];
    const cplx *v = A + (k + 1) + (int64_t)k * lda;
    double sr = 0.0, si = 0.0;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        cplx p = mk(0.0, 0.0);
        for (int c = 0; c < nchunk; c++) p = cadd(p, ppart[(int64_t)c * n + i]);
        cplx x = cmul(t, p);
        w[i] = x;
        cplx xv = cmul(cconj(x), v[i]);
        sr += xv.x;
        si += xv.y;
    }
    sr = eig_block_sum(sr, sh);
    si = eig_block_sum(si, sh);
    cplx alpha = cmul(mk(-0.5, 0.0), cmul(t, mk(sr, si)));
    for (int i = threadIdx.x; i < m; i += blockDim.x) w[i] = cadd(w[i], cmul(alpha, v[i]));
}

// A(k+1:, k+1:) -= v w^H + w v^H
__global__ void hh_update_kernel(int n, int k, cplx *A, int64_t lda, const cplx *w) {
    const int m = n - k - 1;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (i >= m || j >= m) return;
    const cplx *v = A + (k + 1) + (int64_t)k * lda;
    cplx vi = v[i], vj = v[j], wi = w[i], wj = w[j];
    int64_t o = (k + 1 + i) + (int64_t)(k + 1 + j) * lda;
    cplx a = A[o];
    a = csub(a, cmulc(vi, wj));
    a = csub(a, cmulc(wi, vj));
    if (i == j) a.y = 0.0;
    A[o] = a;
}

__global__ void hh_last_kernel(int n, const cplx *A, int64_t lda, double *d) {
    d[n - 1] = A[(n - 1) + (int64_t)(n - 1) * lda].x;
}

// ---- persistent form: one cooperative launch for all columns, two grid barriers per column.
// Every block recomputes the reflector of column k (identical arithmetic in every block) and
// stages v in shared memory; a warp per column computes p = A22 v (A22 Hermitian, so
// p_i = column i of A22, conjugated, dotted with v); after the first barrier every block
// forms w = tau p + alpha v and applies A22 -= v w^H + w v^H to its columns.  Data written by
// other blocks is read with ld.global.cg so no stale L1 line is used.
struct GridBar {
    unsigned count;
    unsigned gen;
    int err;       // 1: a barrier wait exceeded its time limit
    unsigned pub;  // reflectors published so far (shared-memory tridiagonalisation)
    unsigned long long limit_ns;   // time limit of one wait (set by the host before the launch)
};

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier for a cooperative launch: one monotonically increasing arrival counter
// (count), so a barrier costs one fence, one atomic and an acquire poll.  Each wait is bounded
// (gb->limit_ns, 5 s by default, the clock read every 16 polls); a block that gives up sets
// gb->err and every waiting block then leaves the kernel.
constexpr uint64_t kBarrierLimitNs = 5000000000ull;
__device__ __forceinline__ bool grid_barrier(GridBar *gb, unsigned nblocks) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        __threadfence();
        const unsigned arrive = atomicAdd(&gb->count, 1u);
        const unsigned target = (arrive / nblocks + 1u) * nblocks;
        unsigned cur;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(&gb->count) : "memory");
        if ((int)(cur - target) < 0) {
            const uint64_t t0 = globaltimer_ns();
            unsigned spins = 0;
            while (true) {
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(&gb->count) : "memory");
                if ((int)(cur - target) >= 0) break;
                if ((++spins & 15u) == 0) {
                    if (*(volatile int *)&gb->err) {
                        ok = 0;
                        break;
                    }
                    if (globaltimer_ns() - t0 > gb->limit_ns) {
                        atomicExch(&gb->err, 1);
                        ok = 0;
                        break;
                    }
                }
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Wait until gb->pub >= want (a point-to-point signal from one block instead of a grid
// barrier); bounded like grid_barrier.  Ends with __syncthreads.
__device__ __forceinline__ bool wait_published(GridBar *gb, unsigned want) {
    __shared__ int s_ok2;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        unsigned cur;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(&gb->pub) : "memory");
        if (cur < want) {
            const uint64_t t0 = globaltimer_ns();
            unsigned spins = 0;
            while (true) {
                asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(&gb->pub) : "memory");
                if (cur >= want) break;
                if ((++spins & 15u) == 0) {
                    if (*(volatile int *)&gb->err) {
                        ok = 0;
                        break;
                    }
                    if (globaltimer_ns() - t0 > gb->limit_ns) {
                        atomicExch(&gb->err, 1);
                        ok = 0;
                        break;
                    }
                }
            }
        }
        s_ok2 = ok;
    }
    __syncthreads();
    return s_ok2 != 0;
}

// Two deterministic block sums in one pass (sh >= 64 doubles); every thread gets both.
__device__ void eig_block_sum2(double &a, double &b, double *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    __syncthreads();
    if (lane == 0) {
        sh[wid] = a;
        sh[32 + wid] = b;
    }
    __syncthreads();
    if (wid == 0) {
        double x = lane < nw ? sh[lane] : 0.0, y = lane < nw ? sh[32 + lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, o);
            y += __shfl_down_sync(0xffffffffu, y, o);
        }
        if (lane == 0) {
            sh[0] = x;
            sh[32] = y;
        }
    }
    __syncthreads();
    a = sh[0];
    b = sh[32];
}

__device__ __forceinline__ cplx ldcg(const cplx *p) { return __ldcg(p); }

constexpr int TRD_THREADS = 512;
constexpr int TRD_UNROLL = 8;
constexpr int kTridiagPersistentMaxN = 7000;   // v and w staged in shared memory: 32 bytes per row

__global__ void __launch_bounds__(TRD_THREADS) tridiag_persistent_kernel(int n, cplx *A, int64_t lda, double *d,
                                                                         double *e, cplx *tau, cplx *pbuf,
                                                                         double2 *part, GridBar *gb) {
    extern __shared__ cplx tsm[];
    __shared__ double red[32];
    __shared__ cplx s_scale, s_tau, s_alpha;
    __shared__ double s_beta;
    __shared__ int s_skip;
    const unsigned nb = gridDim.x;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    const int gw = blockIdx.x * nwb + wib, nw = nb * nwb;
    cplx *sv = tsm, *sw = tsm + (n > 1 ? n - 1 : 1);
    for (int k = 0; k + 1 < n; k++) {
        const int m = n - k - 1;
        cplx *x = A + (k + 1) + (int64_t)k * lda;
        // reflector of column k (same in every block)
        double ss = 0.0;
        for (int i = 1 + threadIdx.x; i < m; i += blockDim.x) ss += cabs2(ldcg(x + i));
        ss = eig_block_sum(ss, red);
        if (threadIdx.x == 0) {
            const cplx alpha = ldcg(x);
            const double xnorm = sqrt(ss);
            if (xnorm == 0.0 && alpha.y == 0.0) {
                s_tau = mk(0.0, 0.0);
                s_beta = alpha.x;
                s_skip = 1;
                s_scale = mk(1.0, 0.0);
            } else {
                const double nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm * xnorm);
                const double beta = alpha.x >= 0.0 ? -nrm : nrm;
                s_tau = mk((beta - alpha.x) / beta, -alpha.y / beta);
                s_beta = beta;
                s_scale = cdiv(mk(1.0, 0.0), mk(alpha.x - beta, alpha.y));
                s_skip = 0;
            }
        }
        __syncthreads();
        const cplx t = s_tau, sc = s_scale;
        const bool active = !s_skip;
        for (int i = threadIdx.x; i < m; i += blockDim.x) sv[i] = i == 0 ? mk(1.0, 0.0) : (active ? cmul(ldcg(x + i), sc) : ldcg(x + i));
        __syncthreads();
        // p = tau * A22 v (warp per column), partial x^H v with x = tau p
        double pr = 0.0, pim = 0.0;
        if (active) {
            for (int i = gw; i < m; i += nw) {
                const cplx *col = A + (k + 1) + (int64_t)(k + 1 + i) * lda;
                // conj(column) . v with TRD_UNROLL loads in flight per lane (the loop is L2-latency bound)
                double arr[TRD_UNROLL], aii[TRD_UNROLL];
#pragma unroll
                for (int u = 0; u < TRD_UNROLL; u++) arr[u] = aii[u] = 0.0;
                int j = lane;
                for (; j + 32 * (TRD_UNROLL - 1) < m; j += 32 * TRD_UNROLL) {
                    cplx a[TRD_UNROLL];
#pragma unroll
                    for (int u = 0; u < TRD_UNROLL; u++) a[u] = ldcg(col + j + 32 * u);
#pragma unroll
                    for (int u = 0; u < TRD_UNROLL; u++) {
                        const cplx v = sv[j + 32 * u];
                        arr[u] += a[u].x * v.x + a[u].y * v.y;
                        aii[u] += a[u].x * v.y - a[u].y * v.x;
                    }
                }
                for (; j < m; j += 32) {
                    const cplx a = ldcg(col + j), v = sv[j];
                    arr[0] += a.x * v.x + a.y * v.y;
                    aii[0] += a.x * v.y - a.y * v.x;
                }
                double ar = 0.0, ai = 0.0;
#pragma unroll
                for (int u = 0; u < TRD_UNROLL; u++) {
                    ar += arr[u];
                    ai += aii[u];
                }
                for (int o = 16; o > 0; o >>= 1) {
                    ar += __shfl_down_sync(0xffffffffu, ar, o);
                    ai += __shfl_down_sync(0xffffffffu, ai, o);
                }
                if (lane == 0) {
                    const cplx xp = cmul(t, mk(ar, ai));
                    pbuf[i] = xp;
                    const cplx xv = cmul(cconj(xp), sv[i]);
                    pr += xv.x;
                    pim += xv.y;
                }
            }
        }
        pr = eig_block_sum(pr, red);
        pim = eig_block_sum(pim, red);
        if (threadIdx.x == 0) part[blockIdx.x] = make_double2(pr, pim);
        if (!grid_barrier(gb, nb)) return;
        if (active) {
            double sr = 0.0, si = 0.0;
            for (unsigned b = threadIdx.x; b < nb; b += blockDim.x) {
                const double2 q = __ldcg(part + b);
                sr += q.x;
                si += q.y;
            }
            sr = eig_block_sum(sr, red);
            si = eig_block_sum(si, red);
            if (threadIdx.x == 0) s_alpha = cmul(mk(-0.5, 0.0), cmul(t, mk(sr, si)));
            __syncthreads();
            const cplx al = s_alpha;
            for (int i = threadIdx.x; i < m; i += blockDim.x) sw[i] = cadd(ldcg(pbuf + i), cmul(al, sv[i]));
            __syncthreads();
            for (int j = gw; j < m; j += nw) {
                const cplx vj = sv[j], wj = sw[j];
                cplx *col = A + (k + 1) + (int64_t)(k + 1 + j) * lda;
                int i = lane;
                for (; i + 32 * (TRD_UNROLL - 1) < m; i += 32 * TRD_UNROLL) {
                    cplx a[TRD_UNROLL];
#pragma unroll
                    for (int u = 0; u < TRD_UNROLL; u++) a[u] = ldcg(col + i + 32 * u);
#pragma unroll
                    for (int u = 0; u < TRD_UNROLL; u++) {
                        const int r = i + 32 * u;
                        cplx x = csub(a[u], cmulc(sv[r], wj));
                        x = csub(x, cmulc(sw[r], vj));
                        if (r == j) x.y = 0.0;
                        col[r] = x;
                    }
                }
                for (; i < m; i += 32) {
                    cplx a = ldcg(col + i);
                    a = csub(a, cmulc(sv[i], wj));
                    a = csub(a, cmulc(sw[i], vj));
                    if (i == j) a.y = 0.0;
                    col[i] = a;
                }
            }
        }
        if (blockIdx.x == 0) {
            for (int i = threadIdx.x; i < m; i += blockDim.x) x[i] = sv[i];
            if (threadIdx.x == 0) {
                d[k] = ldcg(A + k + (int64_t)k * lda).x;
                e[k] = s_beta;
                tau[k] = t;
            }
        }
        if (!grid_barrier(gb, nb)) return;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) d[n - 1] = ldcg(A + (n - 1) + (int64_t)(n - 1) * lda).x;
}

// ---- shared-memory-resident form (n up to kTridiagSmemMaxN): the matrix lives in the blocks'
// shared memory for the whole reduction, block b owning columns b, b + nb, ...  Per column k
// the global traffic is the reflector v (written by the owner of column k), the all-gathered
// p = tau A22 v (one entry per column, from its owner) and one partial dot per block; the
// matvec and the rank-2 update run from shared memory.  The warp that updates column k+1
// forms the next reflector from it right away and signals it; per column one grid barrier
// (before w) and one wait for the published reflector.
constexpr int kTridiagSmemMaxN = 1400;

// reflector of x[0..m) (x[0] = alpha), by one warp; returns tau, beta, the scale for x[1:]
__device__ __forceinline__ void warp_reflector(const cplx *x, int m, cplx &tau, double &beta, cplx &scale,
                                               bool &skip) {
    const int lane = threadIdx.x & 31;
    double ss = 0.0;
    for (int i = 1 + lane; i < m; i += 32) ss += cabs2(x[i]);
    ss = eig_warp_sum(ss);
    const cplx alpha = x[0];
    const double xnorm = sqrt(ss);
    if (xnorm == 0.0 && alpha.y == 0.0) {
        tau = mk(0.0, 0.0);
        beta = alpha.x;
        scale = mk(1.0, 0.0);
        skip = true;
    } else {
        const double nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xnorm * xnorm);
        beta = alpha.x >= 0.0 ? -nrm : nrm;
        tau = mk((beta - alpha.x) / beta, -alpha.y / beta);
        scale = cdiv(mk(1.0, 0.0), mk(alpha.x - beta, alpha.y));
        skip = false;
    }
}

// Column k+1 is in this block's shared memory (local slot c): write its reflector (rows k+2..)
// to A(k+2:, k+1), and d[k+1], e[k+1], tau[k+1].  One warp.  With pub, the warp then raises
// the published-reflector count to k1 + 1 (release order after every lane's writes).
__device__ __forceinline__ void publish_reflector(int n, int k1, const cplx *col, cplx *A, int64_t lda, double *d,
                                                  double *e, cplx *tau, unsigned *pub = nullptr) {
    const int lane = threadIdx.x & 31;
    const int m = n - k1 - 1;
    const cplx *x = col + k1 + 1;
    cplx t, sc;
    double beta;
    bool skip;
    warp_reflector(x, m, t, beta, sc, skip);
    cplx *g = A + (k1 + 1) + (int64_t)k1 * lda;
    for (int i = lane; i < m; i += 32) g[i] = i == 0 ? mk(1.0, 0.0) : (skip ? x[i] : cmul(x[i], sc));
    if (lane == 0) {
        tau[k1] = t;
        e[k1] = beta;
        d[k1] = col[k1].x;
    }
    if (pub) {
        __threadfence();
        __syncwarp();
        if (lane == 0) atomicMax(pub, (unsigned)(k1 + 1));
    }
}

// One problem of a batched launch: its matrix, outputs, scratch and the block range
// [b0, b0 + nb) that reduces it (with its own grid barrier).
struct TrdJob {
    cplx *A;
    int64_t lda;
    double *d, *e;
    cplx *tau, *pbuf;
    double2 *part;
    GridBar *gb;
    int n, b0, nb;
};

__device__ void tridiag_smem_body(int n, cplx *A, int64_t lda, double *d, double *e, cplx *tau, cplx *pbuf,
                                  double2 *part, GridBar *gb, const int b, const unsigned nb) {
    extern __shared__ cplx tsm2[];
    __shared__ double red[64];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    const int nown = (n - b + (int)nb - 1) / (int)nb;   // columns b, b+nb, ...
    cplx *cols = tsm2;                                    // nown x n
    cplx *sv = cols + (size_t)nown * n, *sw = sv + n;
    for (int64_t x = threadIdx.x; x < (int64_t)nown * n; x += blockDim.x) {
        const int c = (int)(x / n), r = (int)(x % n);
        cols[x] = A[r + (int64_t)(b + c * (int)nb) * lda];
    }
    __syncthreads();
    if (b == 0 && wib == 0) {
        if (n >= 2) publish_reflector(n, 0, cols, A, lda, d, e, tau, &gb->pub);
        else if (lane == 0) d[0] = cols[0].x;
    }
    for (int k = 0; k + 1 < n; k++) {
        // reflector k, published by the owner of column k (the only dependency on the
        // previous column): a point-to-point wait instead of a second grid barrier.  The
        // p / partial buffers alternate by parity, so a block that starts column k+1 early
        // cannot overwrite what a slower block still reads for column k.
        if (!wait_published(gb, (unsigned)(k + 1))) return;
        cplx *pb = pbuf + (size_t)(k & 1) * (n + 1);
        double2 *pt = part + (size_t)(k & 1) * (n + 1);   // per-column terms conj(p_j) v_j
        const cplx t = ldcg(tau + k);
        const bool active = (t.x != 0.0 || t.y != 0.0);
        for (int r = k + 1 + threadIdx.x; r < n; r += blockDim.x) sv[r] = ldcg(A + r + (int64_t)k * lda);
        __syncthreads();
        // first owned column index > k
        const int c0 = k + 1 > b ? (k + 1 - b + (int)nb - 1) / (int)nb : 0;
        if (active) {
            for (int c = c0 + wib; c < nown; c += nwb) {
                const int j = b + c * (int)nb;
                const cplx *col = cols + (size_t)c * n;
                double ar = 0.0, ai = 0.0;
                for (int r = k + 1 + lane; r < n; r += 32) {
                    const cplx a = col[r], v = sv[r];
                    ar += a.x * v.x + a.y * v.y;
                    ai += a.x * v.y - a.y * v.x;
                }
                for (int o = 16; o > 0; o >>= 1) {
                    ar += __shfl_down_sync(0xffffffffu, ar, o);
                    ai += __shfl_down_sync(0xffffffffu, ai, o);
                }
                if (lane == 0) {
                    const cplx xp = cmul(t, mk(ar, ai));
                    pb[j] = xp;
                    const cplx xv = cmul(cconj(xp), sv[j]);
                    pt[j] = make_double2(xv.x, xv.y);
                }
            }
        }
        if (!grid_barrier(gb, nb)) return;
        if (active) {
            // p^H v summed over the columns in a fixed order (thread stride, then the block
            // sum): the same bits whatever the number of blocks reducing this matrix
            double sr = 0.0, si = 0.0;
            for (int q = k + 1 + threadIdx.x; q < n; q += blockDim.x) {
                const double2 v = __ldcg(pt + q);
                sr += v.x;
                si += v.y;
            }
            eig_block_sum2(sr, si, red);
            const cplx al = cmul(mk(-0.5, 0.0), cmul(t, mk(sr, si)));
            for (int r = k + 1 + threadIdx.x; r < n; r += blockDim.x) sw[r] = cadd(ldcg(pb + r), cmul(al, sv[r]));
            __syncthreads();
        }
        // update owned columns > k; the warp that owns column k+1 then publishes its reflector
        for (int c = c0 + wib; c < nown; c += nwb) {
            const int j = b + c * (int)nb;
            cplx *col = cols + (size_t)c * n;
            if (active) {
                const cplx vj = sv[j], wj = sw[j];
                for (int r = k + 1 + lane; r < n; r += 32) {
                    // a -= v_r conj(w_j) + w_r conj(v_j), as eight FMAs
                    const cplx vr = sv[r], wr = sw[r];
                    cplx a = col[r];
                    a.x = fma(-vr.x, wj.x, a.x);
                    a.x = fma(-vr.y, wj.y, a.x);
                    a.x = fma(-wr.x, vj.x, a.x);
                    a.x = fma(-wr.y, vj.y, a.x);
                    a.y = fma(-vr.y, wj.x, a.y);
                    a.y = fma(vr.x, wj.y, a.y);
                    a.y = fma(-wr.y, vj.x, a.y);
                    a.y = fma(wr.x, vj.y, a.y);
                    if (r == j) a.y = 0.0;
                    col[r] = a;
                }
                __syncwarp();
            }
            if (j == k + 1) {
                if (k + 2 < n) publish_reflector(n, k + 1, col, A, lda, d, e, tau, &gb->pub);
                else if (lane == 0) d[k + 1] = col[k + 1].x;
            }
        }
    }
}

// ---- cluster form (n up to kTridiagClusterMaxN): the same column-cyclic reduction within one
// thread-block cluster per matrix, the blocks exchanging through distributed shared memory
// instead of L2.  The owner of column k keeps its reflector and tau in its shared memory;
// each block keeps the p_j and conj(p_j) v_j of its own columns there; the others read
// them with loads from the owner's shared-memory window.  The synchronisation (one barrier
// and one published-reflector wait per column) runs on counters in shared memory, with
// cluster-scope release and acquire: a few hundred cycles instead of L2 round trips, which
// set the column time of small matrices in the cooperative form.  The arithmetic and every
// summation order are those of tridiag_smem_body, so both give the same bits.
constexpr int kTridiagClusterMaxN = 400;

// generic address of the same shared-memory location in cluster block `rank`
template <class T>
__device__ __forceinline__ T *cl_map(T *p, unsigned rank) {
    return static_cast<T *>(__cluster_map_shared_rank(static_cast<const void *>(p), rank));
}
__device__ __forceinline__ void cl_sync_all() {
    __cluster_barrier_arrive();
    __cluster_barrier_wait();
}
__device__ __forceinline__ unsigned cl_ld_acquire(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.cluster.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void cl_max_relaxed(unsigned *p, unsigned x) {
    asm volatile("red.relaxed.cluster.max.u32 [%0], %1;" ::"l"(p), "r"(x) : "memory");
}
__device__ __forceinline__ void cl_fence() { asm volatile("fence.acq_rel.cluster;" ::: "memory"); }

// One thread: wait until *p >= want, bounded like grid_barrier (gb->limit_ns, gb->err).
__device__ bool cl_wait_geq(const unsigned *p, unsigned want, GridBar *gb) {
    if ((int)(cl_ld_acquire(p) - want) >= 0) return true;
    const uint64_t t0 = globaltimer_ns();
    unsigned spins = 0;
    while (true) {
        if ((int)(cl_ld_acquire(p) - want) >= 0) return true;
        if ((++spins & 15u) == 0) {
            if (*(volatile int *)&gb->err) return false;
            if (globaltimer_ns() - t0 > gb->limit_ns) {
                atomicExch(&gb->err, 1);
                return false;
            }
        }
    }
}

// Cluster-wide barrier: every block adds its arrival to the counter of every block (bar, its
// own shared counter, mapped), then waits on its own copy, so the polling stays in local
// shared memory instead of loading another block's; `gen` counts the barriers passed.
__device__ __forceinline__ void cl_add_relaxed(unsigned *p, unsigned x) {
    asm volatile("red.relaxed.cluster.add.u32 [%0], %1;" ::"l"(p), "r"(x) : "memory");
}
__device__ bool cl_barrier(unsigned *bar, unsigned ncta, unsigned gen, GridBar *gb, int *s_ok) {
    __syncthreads();
    if (threadIdx.x == 0) {
        cl_fence();   // the block's writes before the arrivals (one fence, then plain reductions)
        for (unsigned r = 0; r < ncta; r++) cl_add_relaxed(cl_map(bar, r), 1u);
        *s_ok = cl_wait_geq(bar, (gen + 1u) * ncta, gb);
    }
    __syncthreads();
    return *s_ok != 0;
}

// publish_reflector for the cluster form: the reflector also goes to the owner's shared copy
// vl (indexed by row) and tau to *stau, then the published count k1 + 1 to every block's own
// counter (pub, mapped per block), where the waiters poll it locally.
__device__ __forceinline__ void publish_reflector_cl(int n, int k1, const cplx *col, cplx *A, int64_t lda,
                                                     double *d, double *e, cplx *tau, cplx *vl, cplx *stau,
                                                     unsigned *pub, unsigned ncta) {
    const int lane = threadIdx.x & 31;
    const int m = n - k1 - 1;
    const cplx *x = col + k1 + 1;
    cplx t, sc;
    double beta;
    bool skip;
    warp_reflector(x, m, t, beta, sc, skip);
    cplx *g = A + (k1 + 1) + (int64_t)k1 * lda;
    for (int i = lane; i < m; i += 32) {
        const cplx v = i == 0 ? mk(1.0, 0.0) : (skip ? x[i] : cmul(x[i], sc));
        g[i] = v;
        vl[k1 + 1 + i] = v;
    }
    if (lane == 0) {
        tau[k1] = t;
        e[k1] = beta;
        d[k1] = col[k1].x;
        *stau = t;
    }
    __syncwarp();
    if (lane == 0) {
        cl_fence();   // the warp's writes before the counts
        for (unsigned r = 0; r < ncta; r++) cl_max_relaxed(cl_map(pub, r), (unsigned)(k1 + 1));
    }
}

// Dynamic shared memory of one cluster block: two parities of the published reflector and of
// the block's own p and conj(p) v (compact, by owned column), then v, w and the gathered p and
// conj(p) v of all columns (10 rows of n complex), then its columns.
static size_t trd_cluster_bytes(int n, int ncta) { return (size_t)(((n + ncta - 1) / ncta) + 10) * n * sizeof(cplx); }

// Blocks per cluster for an order-n matrix (a function of n alone, so a matrix reduces the
// same way whichever batch it is in): more blocks share the FP64 work of larger matrices,
// fewer keep the synchronisation short for small ones.
static int trd_cluster_ctas(int n) {
    if (n <= 32) return 1;
    if (n <= 64) return 4;
    return 16;   // a GB300 SM retires two FP64 FMAs per clock: the column work needs the blocks
}

__global__ void __launch_bounds__(TRD_THREADS) tridiag_cluster_kernel(const TrdJob *__restrict__ jobs, int njobs,
                                                                       int ncta_expect, unsigned smem_bytes,
                                                                       int *status) {
    extern __shared__ cplx tsm3[];
    __shared__ double red[64];
    __shared__ unsigned s_bar, s_pub;
    __shared__ cplx s_tau[2];
    __shared__ int s_ok;
    const unsigned ncta = __clusterSizeInBlocks();
    const int b = (int)__clusterRelativeBlockRank();
    // launch-shape checks, the same for every block of a cluster (none touches another block
    // before they pass): a cluster of the expected size, a job per cluster, and room for the
    // job's columns in the dynamic shared memory
    if ((int)ncta != ncta_expect || gridDim.x != ncta * (unsigned)njobs) {
        if (threadIdx.x == 0) atomicCAS(status, 0, 1);
        return;
    }
    const TrdJob J = jobs[blockIdx.x / ncta];
    const int n = J.n, nb = (int)ncta;
    if (n < 1 || nb > TRD_THREADS / 32 || (size_t)(((n + nb - 1) / nb) + 10) * n * sizeof(cplx) > smem_bytes) {
        if (threadIdx.x == 0) atomicCAS(status, 0, 2);
        return;
    }
    cplx *A = J.A;
    const int64_t lda = J.lda;
    GridBar *gb = J.gb;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, nwb = blockDim.x >> 5;
    const int nown = (n - b + nb - 1) / nb;   // columns b, b+nb, ...
    // the buffers other blocks read come first, at the same offsets in every block (a mapped
    // address is the same offset in another block); the block's own columns (a count that
    // differs between blocks) come last
    cplx *vloc = tsm3;                        // 2 x n: published reflector by parity
    cplx *pbl = vloc + 2 * (size_t)n;         // 2 x n: p_j of own column slot c at [par n + c]
    double2 *ptl = reinterpret_cast<double2 *>(pbl + 2 * (size_t)n);   // 2 x n: conj(p_j) v_j, same
    cplx *sv = reinterpret_cast<cplx *>(ptl + 2 * (size_t)n), *sw = sv + n;
    cplx *pall = sw + n;                      // p_j of every column, gathered
    double2 *ptall = reinterpret_cast<double2 *>(pall + n);   // conj(p_j) v_j of every column
    cplx *cols = reinterpret_cast<cplx *>(ptall + n);         // nown x n
    if (threadIdx.x == 0) {
        s_bar = 0;
        s_pub = 0;
    }
    for (int64_t x = threadIdx.x; x < (int64_t)nown * n; x += blockDim.x) {
        const int c = (int)(x / n), r = (int)(x % n);
        cols[x] = A[r + (int64_t)(b + c * nb) * lda];
    }
    __syncthreads();
    cl_sync_all();   // every block's counters set before any other block touches them
    unsigned gen = 0;   // cluster barriers passed
    if (b == 0 && wib == 0) {
        if (n >= 2) publish_reflector_cl(n, 0, cols, A, lda, J.d, J.e, J.tau, vloc, &s_tau[0], &s_pub, ncta);
        else if (lane == 0) J.d[0] = cols[0].x;
    }
    for (int k = 0; k + 1 < n; k++) {
        const unsigned owner = (unsigned)(k % nb);
        if (threadIdx.x == 0) s_ok = cl_wait_geq(&s_pub, (unsigned)(k + 1), gb);
        __syncthreads();
        if (!s_ok) break;
        const int par = k & 1;
        const cplx t = *cl_map(&s_tau[par], owner);
        const bool active = (t.x != 0.0 || t.y != 0.0);
        {
            const cplx *vr = cl_map(vloc + (size_t)par * n, owner);
            for (int r = k + 1 + threadIdx.x; r < n; r += blockDim.x) sv[r] = vr[r];
        }
        __syncthreads();
        cplx *pb = pbl + (size_t)par * n;
        double2 *pt = ptl + (size_t)par * n;
        const int c0 = k + 1 > b ? (k + 1 - b + nb - 1) / nb : 0;
        if (active) {
            for (int c = c0 + wib; c < nown; c += nwb) {
                const int j = b + c * nb;
                const cplx *col = cols + (size_t)c * n;
                double ar = 0.0, ai = 0.0;
                for (int r = k + 1 + lane; r < n; r += 32) {
                    const cplx a = col[r], v = sv[r];
                    ar += a.x * v.x + a.y * v.y;
                    ai += a.x * v.y - a.y * v.x;
                }
                for (int o = 16; o > 0; o >>= 1) {
                    ar += __shfl_down_sync(0xffffffffu, ar, o);
                    ai += __shfl_down_sync(0xffffffffu, ai, o);
                }
                if (lane == 0) {
                    const cplx xp = cmul(t, mk(ar, ai));
                    pb[c] = xp;
                    const cplx xv = cmul(cconj(xp), sv[j]);
                    pt[c] = make_double2(xv.x, xv.y);
                }
            }
        }
        if (!cl_barrier(&s_bar, ncta, gen++, gb, &s_ok)) break;
        if (active) {
            // gather: warp o reads block o's compact values (contiguous, one block per warp)
            if (wib < nb) {
                const int o = wib, no = (n - o + nb - 1) / nb;
                const int co = k + 1 > o ? (k + 1 - o + nb - 1) / nb : 0;
                const cplx *rpb = cl_map(pb, (unsigned)o);
                const double2 *rpt = cl_map(pt, (unsigned)o);
                for (int c = co + lane; c < no; c += 32) {
                    const int j = o + c * nb;
                    pall[j] = rpb[c];
                    ptall[j] = rpt[c];
                }
            }
            __syncthreads();
            double sr = 0.0, si = 0.0;
            for (int q = k + 1 + threadIdx.x; q < n; q += blockDim.x) {
                const double2 v = ptall[q];
                sr += v.x;
                si += v.y;
            }
            eig_block_sum2(sr, si, red);
            const cplx al = cmul(mk(-0.5, 0.0), cmul(t, mk(sr, si)));
            for (int r = k + 1 + threadIdx.x; r < n; r += blockDim.x) sw[r] = cadd(pall[r], cmul(al, sv[r]));
            __syncthreads();
        }
        for (int c = c0 + wib; c < nown; c += nwb) {
            const int j = b + c * nb;
            cplx *col = cols + (size_t)c * n;
            if (active) {
                const cplx vj = sv[j], wj = sw[j];
                for (int r = k + 1 + lane; r < n; r += 32) {
                    const cplx vr = sv[r], wr = sw[r];
                    cplx a = col[r];
                    a.x = fma(-vr.x, wj.x, a.x);
                    a.x = fma(-vr.y, wj.y, a.x);
                    a.x = fma(-wr.x, vj.x, a.x);
                    a.x = fma(-wr.y, vj.y, a.x);
                    a.y = fma(-vr.y, wj.x, a.y);
                    a.y = fma(vr.x, wj.y, a.y);
                    a.y = fma(-wr.y, vj.x, a.y);
                    a.y = fma(wr.x, vj.y, a.y);
                    if (r == j) a.y = 0.0;
                    col[r] = a;
                }
                __syncwarp();
            }
            if (j == k + 1) {
                if (k + 2 < n)
                    publish_reflector_cl(n, k + 1, col, A, lda, J.d, J.e, J.tau, vloc + (size_t)((k + 1) & 1) * n,
                                         &s_tau[(k + 1) & 1], &s_pub, ncta);
                else if (lane == 0) J.d[k + 1] = col[k + 1].x;
            }
        }
    }
    cl_sync_all();   // no block leaves while another may still read its shared memory
}

// Batched tridiagonalisation: several Hermitian matrices in one cooperative launch, each
// reduced by its own group of blocks, so the barrier-bound column loops of independent
// problems overlap instead of running one after another.
__global__ void __launch_bounds__(TRD_THREADS) tridiag_smem_batched_kernel(const TrdJob *__restrict__ jobs,
                                                                            int njobs) {
    int j = 0;
    while (j + 1 < njobs && (int)blockIdx.x >= jobs[j + 1].b0) j++;
    const TrdJob J = jobs[j];
    tridiag_smem_body(J.n, J.A, J.lda, J.d, J.e, J.tau, J.pbuf, J.part, J.gb, (int)blockIdx.x - J.b0,
                      (unsigned)J.nb);
}

// ===================================================================== 2. divide and conquer
// Per-level scratch, every array of length n and sliced by node (a node owns [s, s+N)).
struct DcBufs {
    double *lamA, *lamB;      // eigenvalues of the current / next level
    double *QA, *QB;          // eigenvector matrices (n x n, ld n), block diagonal by node
    double *U;                // merge eigenvector matrices, block diagonal (n x n, ld n)
    double *dK, *zK;          // undeflated poles and rank-one components (compact, per node)
    double *dv;               // deflated eigenvalues (per node)
    int *Kl, *defl;           // node-local column of each undeflated / deflated entry
    int *rp, *rn;             // Givens rotation column pairs
    double *rc, *rs;          // and their cosines / sines
    int *ord;                 // origin pole of each secular root
    double *tau, *lamK;       // root offset from its origin, root value
    double *zh;               // recomputed rank-one vector
    int *outc;                // output column of each node entry in the next level
    int *kcnt, *ndef, *nrot;  // per node: undeflated count (-1: pass-through), deflated, rotations
    double *rho;              // per node
    int *status;              // nonzero: a merge met an inconsistent pole order
};

__global__ void dc_leaf_kernel(int n, const double *__restrict__ d, const double *__restrict__ e, double *lam,
                               double *Q) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = d[i];
    if (i > 0) v -= fabs(e[i - 1]);
    if (i < n - 1) v -= fabs(e[i]);
    lam[i] = v;
    Q[i + (int64_t)i * n] = 1.0;
}

// Exclusive block prefix sum of one int per thread (blockDim.x <= 1024); total gets the sum.
// Every thread of the block must call it.
__device__ int dc_block_excl_scan(int v, int *wsum, int &total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    if (wid == 0) {
        int t = lane < nw ? wsum[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        __syncwarp();
        wsum[lane] = t;
    }
    __syncthreads();
    total = wsum[nw - 1];
    const int base = (wid > 0 ? wsum[wid - 1] : 0) + x - v;
    __syncthreads();
    return base;
}

// One block per node: rank-one vector, merge order, deflation (in parallel, or thread 0
// scanning the merged order when a pair rotation is due), rotations applied to the node's
// eigenvector columns.  Dynamic shared memory: 20 bytes per node column.
__global__ void dc_prep_kernel(int n, int half, int full, const double *__restrict__ e, DcBufs b) {
    extern __shared__ double smem[];
    __shared__ double red[32];
    const int node = blockIdx.x;
    const int s = node * full;
    const int N = min(full, n - s);
    const int n1 = half, n2 = N - half;
    if (n2 <= 0) {   // no right sibling at this level: carry the block over
        for (int i = threadIdx.x; i < N; i += blockDim.x) b.lamB[s + i] = b.lamA[s + i];
        for (int64_t x = threadIdx.x; x < (int64_t)N * N; x += blockDim.x) {
            const int r = (int)(x % N), cc = (int)(x / N);
            b.QB[(s + r) + (int64_t)(s + cc) * n] = b.QA[(s + r) + (int64_t)(s + cc) * n];
        }
        if (threadIdx.x == 0) b.kcnt[node] = -1;
        return;
    }
    double *sd = smem, *sz = smem + N;
    int *sp = reinterpret_cast<int *>(smem + 2 * N);
    const double beta = e[s + n1 - 1];
    const double rho = 2.0 * fabs(beta);
    const double sg = beta < 0.0 ? -1.0 : 1.0;
    double mx = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        sd[i] = b.lamA[s + i];
        const double q = i < n1 ? b.QA[(s + n1 - 1) + (int64_t)(s + i) * n] : sg * b.QA[(s + n1) + (int64_t)(s + i) * n];
        sz[i] = q * 0.70710678118654752440;
        mx = fmax(mx, fmax(fabs(sd[i]), fabs(sz[i])));
    }
    // a valid permutation first: the merge below writes every slot exactly once for ordered
    // inputs, and with unordered ones (NaN) no slot is left holding an index out of range
    for (int i = threadIdx.x; i < N; i += blockDim.x) sp[i] = i;
    const double tol = 8.0 * kUnitRoundoff * eig_block_max(mx, red);   // syncs the block
    // stable merge of the two ascending halves
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        const double v = sd[i];
        int lo, hi;
        if (i < n1) {   // count right entries strictly below v
            lo = n1;
            hi = N;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (sd[mid] < v) lo = mid + 1;
                else hi = mid;
            }
            sp[i + (lo - n1)] = i;
        } else {        // count left entries at or below v
            lo = 0;
            hi = n1;
            while (lo < hi) {
                int mid = (lo + hi) >> 1;
                if (sd[mid] <= v) lo = mid + 1;
                else hi = mid;
            }
            sp[(i - n1) + lo] = i;
        }
    }
    __syncthreads();
    // Deflation, first in parallel: the z test of every entry, the compaction of the kept and
    // deflated lists (a block scan over contiguous chunks of the merged order) and the
    // rotation test of every neighbouring kept pair on the unrotated values.  When no pair
    // qualifies for a rotation (the usual case) these lists are exactly the serial scan's; when
    // one does, thread 0 runs the serial scan below, since a rotation changes later tests.  One
    // thread scanning N entries costs N dependent FP64 chains on a unit that retires two
    // operations per clock per SM.
    __shared__ int s_wsum[32], s_rot;
    {
        const int per = (N + (int)blockDim.x - 1) / (int)blockDim.x;
        const int t0 = min(N, (int)threadIdx.x * per), t1 = min(N, t0 + per);
        int cnt = 0;
        for (int t = t0; t < t1; t++) cnt += !(rho * fabs(sz[sp[t]]) <= tol);
        int total;
        int kb = dc_block_excl_scan(cnt, s_wsum, total);
        for (int t = t0; t < t1; t++) {
            const int nj = sp[t];
            if (!(rho * fabs(sz[nj]) <= tol)) b.Kl[s + kb++] = nj;
            else b.defl[s + (t - kb)] = nj;
        }
        if (threadIdx.x == 0) s_rot = 0;
        __syncthreads();
        int rot = 0;
        for (int m = 1 + (int)threadIdx.x; m < total; m += blockDim.x) {
            const int pj = b.Kl[s + m - 1], nj = b.Kl[s + m];
            double S = sz[pj], C = sz[nj];
            const double tt = hypot(C, S);
            const double T = sd[nj] - sd[pj];
            C /= tt;
            S = -S / tt;
            rot |= fabs(T * C * S) <= tol;
        }
        if (rot) atomicOr(&s_rot, 1);
        __syncthreads();
        if (threadIdx.x == 0 && !s_rot) {
            b.kcnt[node] = total;
            b.ndef[node] = N - total;
            b.nrot[node] = 0;
            b.rho[node] = rho;
        }
    }
    if (threadIdx.x == 0 && s_rot) {
        int kc = 0, nd = 0, nr = 0, pj = -1;
        for (int t = 0; t < N; t++) {
            const int nj = sp[t];
            if (rho * fabs(sz[nj]) <= tol) {
                b.defl[s + nd++] = nj;
                continue;
            }
            if (pj >= 0) {
                double S = sz[pj], C = sz[nj];
                const double tt = hypot(C, S);
                const double T = sd[nj] - sd[pj];
                C /= tt;
                S = -S / tt;
                if (fabs(T * C * S) <= tol) {
                    sz[nj] = tt;
                    sz[pj] = 0.0;
                    b.rp[s + nr] = pj;
                    b.rn[s + nr] = nj;
                    b.rc[s + nr] = C;
                    b.rs[s + nr] = S;
                    nr++;
                    const double dp = sd[pj], dn = sd[nj];
                    sd[pj] = dp * C * C + dn * S * S;
                    sd[nj] = dp * S * S + dn * C * C;
                    b.defl[s + nd++] = pj;
                    kc--;
                }
            }
            b.Kl[s + kc++] = nj;
            pj = nj;
        }
        b.kcnt[node] = kc;
        b.ndef[node] = nd;
        b.nrot[node] = nr;
        b.rho[node] = rho;
    }
    __syncthreads();
    const int kc = b.kcnt[node], nd = b.ndef[node], nr = b.nrot[node];
    for (int m = threadIdx.x; m < kc; m += blockDim.x) {
        const int j = b.Kl[s + m];
        b.dK[s + m] = sd[j];
        b.zK[s + m] = sz[j];
    }
    for (int m = threadIdx.x; m < nd; m += blockDim.x) b.dv[s + m] = sd[b.defl[s + m]];
    if (nr > 0)
        for (int r = threadIdx.x; r < N; r += blockDim.x) {
            double *row = b.QA + (s + r);
            for (int q = 0; q < nr; q++) {
                const int64_t op = (int64_t)(s + b.rp[s + q]) * n, on = (int64_t)(s + b.rn[s + q]) * n;
                const double C = b.rc[s + q], S = b.rs[s + q];
                const double x = row[op], y = row[on];
                row[op] = C * x + S * y;
                row[on] = C * y - S * x;
            }
        }
}

// One warp per secular root: root j of 1/rho + sum_i z_i^2 / (d_i - lambda) = 0 lies in
// (d_j, d_{j+1}) (the last one in (d_{k-1}, d_{k-1} + rho |z|^2)).  It is found as an offset
// tau from the nearer pole d_o, so that d_i - lambda = (d_i - d_o) - tau keeps full
// accuracy.  Each step fits c + s1/(dL - x) + s2/(dR - x) to the value and slope of the two
// partial sums at tau and takes that model's root; steps leaving the bracket bisect.
// All lanes hold identical scalars (lane 0's sums are broadcast), so the warp stays uniform.
__global__ void dc_secular_kernel(int n, int full, DcBufs b) {
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n) return;
    const int node = w / full, s = node * full, j = w - s;
    const int k = b.kcnt[node];
    if (k < 0 || j >= k) return;
    const double *dk = b.dK + s, *zk = b.zK + s;
    const double rho = b.rho[node], rhoinv = 1.0 / rho;
    int o;
    double lo, hi;
    if (j < k - 1) {
        const double dl = dk[j], dr = dk[j + 1];
        if (!(dr > dl)) {
            if (lane == 0) {
                atomicExch(b.status, 1);
                b.ord[s + j] = j;
                b.tau[s + j] = 0.0;
                b.lamK[s + j] = dl;
            }
            return;
        }
        const double hg = 0.5 * (dr - dl);
        double p = 0.0;
        for (int i = lane; i < k; i += 32) p += zk[i] * zk[i] / ((dk[i] - dl) - hg);
        const double g = rhoinv + eig_warp_sum(p);
        if (g > 0.0) {
            o = j;
            lo = 0.0;
            hi = hg;
        } else {
            o = j + 1;
            lo = -hg;
            hi = 0.0;
        }
    } else {
        double p = 0.0;
        for (int i = lane; i < k; i += 32) p += zk[i] * zk[i];
        o = j;
        lo = 0.0;
        hi = rho * eig_warp_sum(p);
    }
    const double d_o = dk[o];
    const int L = j, R = j + 1;
    const double dL = dk[L] - d_o, dR = R < k ? dk[R] - d_o : 0.0;
    double tau = 0.5 * (lo + hi);
    for (int it = 0; it < kSecularMaxIter; it++) {
        double ps = 0.0, ph = 0.0, dps = 0.0, dph = 0.0;
        for (int i = lane; i < k; i += 32) {
            // one division per pole (a GB300 FP64 division is a chain of FP64 operations on a
            // unit that retires two per clock per SM): t = z^2 / den and t / den from 1 / den
            const double r = 1.0 / ((dk[i] - d_o) - tau);
            const double t = zk[i] * zk[i] * r;
            if (i <= L) {
                ps += t;
                dps += t * r;
            } else {
                ph += t;
                dph += t * r;
            }
        }
        ps = eig_warp_sum(ps);
        ph = eig_warp_sum(ph);
        dps = eig_warp_sum(dps);
        dph = eig_warp_sum(dph);
        const double g = rhoinv + ps + ph;
        const double err = 8.0 * (ph - ps) + rhoinv + fabs(tau) * (dps + dph);
        if (fabs(g) <= 4.0 * kUnitRoundoff * err * k) break;
        if (hi - lo <= 2.0 * kUnitRoundoff * fmax(fabs(lo), fabs(hi))) break;
        if (g < 0.0) lo = tau;
        else hi = tau;
        const double s1 = dps * (dL - tau) * (dL - tau);
        double cc = rhoinv + ps - s1 / (dL - tau);
        double x;
        if (R < k) {
            const double s2 = dph * (dR - tau) * (dR - tau);
            cc += ph - s2 / (dR - tau);
            const double A = cc, B = cc * (dL + dR) + s1 + s2, C = cc * dL * dR + s1 * dR + s2 * dL;
            if (A == 0.0) {
                x = C / B;
            } else {
                const double disc = fmax(B * B - 4.0 * A * C, 0.0);
                const double q = 0.5 * (B + copysign(sqrt(disc), B));
                const double r1 = q / A;
                const double r2 = q != 0.0 ? C / q : NAN;
                x = (r1 > lo && r1 < hi) ? r1 : r2;
            }
        } else {
            x = cc > 0.0 ? dL + s1 / cc : NAN;
        }
        if (!(x > lo && x < hi)) x = 0.5 * (lo + hi);
        tau = x;
    }
    if (lane == 0) {
        b.ord[s + j] = o;
        b.tau[s + j] = tau;
        b.lamK[s + j] = d_o + tau;
    }
}

// One warp per undeflated entry i: zhat_i^2 = prod_j |d_i - lambda_j| / prod_{j != i} |d_i - d_j|
// (up to the common factor 1/rho, which the normalisation removes); sign of z_i.
__global__ void dc_zhat_kernel(int n, int full, DcBufs b) {
    const int w = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (w >= n) return;
    const int node = w / full, s = node * full, i = w - s;
    const int k = b.kcnt[node];
    if (k < 0 || i >= k) return;
    const double *dk = b.dK + s;
    const double di = dk[i];
    double p = 1.0;
    for (int j = lane; j < k; j += 32) {
        const double dl = fabs((di - dk[b.ord[s + j]]) - b.tau[s + j]);
        p *= (j == i) ? dl : dl / fabs(dk[j] - di);
    }
    p = eig_warp_prod(p);
    if (lane == 0) b.zh[s + i] = copysign(sqrt(p), b.zK[s + i]);
}

// One warp per node entry: the rank of its eigenvalue in the merged ascending order
// (ties by entry index) gives its column in the next level.
__global__ void dc_rank_kernel(int n, int full, DcBufs b) {
    // one warp per entry (the N comparisons are FP64 operations: one thread per entry left a
    // 792-entry merge on four SMs); every exit below is uniform over the warp
    const int g = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (g >= n) return;
    const int node = g / full, s = node * full, i = g - s;
    const int k = b.kcnt[node];
    if (k < 0) return;
    const int N = k + b.ndef[node];
    if (i >= N) return;
    const double v = i < k ? b.lamK[s + i] : b.dv[s + i - k];
    int r = 0;
    for (int m = lane; m < N; m += 32) {
        const double u = m < k ? b.lamK[s + m] : b.dv[s + m - k];
        r += (u < v) || (u == v && m < i);
    }
    r = __reduce_add_sync(0xffffffffu, r);
    if (lane == 0) {
        b.lamB[s + r] = v;
        b.outc[s + i] = s + r;
    }
}

// One block per node entry: column of the merge eigenvector matrix (undeflated entries),
// or the copy of a deflated eigenvector into its output column.
__global__ void dc_vec_kernel(int n, int full, DcBufs b) {
    __shared__ double red[32];
    const int g = blockIdx.x;
    const int node = g / full, s = node * full, i = g - s;
    const int k = b.kcnt[node];
    if (k < 0) return;
    const int N = k + b.ndef[node];
    if (i >= N) return;
    if (i < k) {
        const double *dk = b.dK + s;
        const double dO = dk[b.ord[s + i]], t = b.tau[s + i];
        double ss = 0.0;
        for (int m = threadIdx.x; m < k; m += blockDim.x) {
            const double u = b.zh[s + m] / ((dk[m] - dO) - t);
            ss += u * u;
        }
        const double inv = 1.0 / sqrt(eig_block_sum(ss, red));
        for (int m = threadIdx.x; m < k; m += blockDim.x)
            b.U[(s + m) + (int64_t)(s + i) * n] = b.zh[s + m] / ((dk[m] - dO) - t) * inv;
    } else {
        const int64_t src = (int64_t)(s + b.defl[s + i - k]) * n, dst = (int64_t)b.outc[s + i] * n;
        for (int r = threadIdx.x; r < N; r += blockDim.x) b.QB[(s + r) + dst] = b.QA[(s + r) + src];
    }
}

// QB(rows of node, outc[j]) = QA(rows of node, Kl[m]) * U(m, j) for the undeflated entries:
// one 64x64 output tile per block, batched over nodes (blockIdx.z).
constexpr int DG_T = 64, DG_K = 16;
__global__ void __launch_bounds__(256) dc_gemm_kernel(int n, int full, DcBufs b) {
    __shared__ double As[DG_K][DG_T + 1];
    __shared__ double Bs[DG_K][DG_T + 1];
    const int node = blockIdx.z, s = node * full;
    const int k = b.kcnt[node];
    if (k <= 0) return;
    const int N = min(full, n - s);
    const int r0 = blockIdx.x * DG_T, c0 = blockIdx.y * DG_T;
    if (r0 >= N || c0 >= k) return;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4] = {};
    for (int m0 = 0; m0 < k; m0 += DG_K) {
        for (int x = threadIdx.x; x < DG_T * DG_K; x += 256) {
            const int rr = x % DG_T, kk = x / DG_T;
            const int gr = r0 + rr, gm = m0 + kk;
            As[kk][rr] = (gr < N && gm < k) ? b.QA[(s + gr) + (int64_t)(s + b.Kl[s + gm]) * n] : 0.0;
        }
        for (int x = threadIdx.x; x < DG_T * DG_K; x += 256) {
            const int kk = x % DG_K, cc = x / DG_K;
            const int gm = m0 + kk, gc = c0 + cc;
            Bs[kk][cc] = (gm < k && gc < k) ? b.U[(s + gm) + (int64_t)(s + gc) * n] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < DG_K; kk++) {
            double a[4], bb[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                a[q] = As[kk][ty + 16 * q];
                bb[q] = Bs[kk][tx + 16 * q];
            }
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++) acc[p][q] = fma(a[p], bb[q], acc[p][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const int gc = c0 + tx + 16 * q;
        if (gc >= k) continue;
        const int64_t col = (int64_t)b.outc[s + gc] * n;
#pragma unroll
        for (int p = 0; p < 4; p++) {
            const int gr = r0 + ty + 16 * p;
            if (gr < N) b.QB[(s + gr) + col] = acc[p][q];
        }
    }
}

// Largest divide-and-conquer dimension: the merge scan keeps 20 bytes per column in shared
// memory (227 KB per block).
constexpr int kDcMaxN = 11264;

static std::string slot_name(const char *base, int slot) { return std::string(base) + "#" + std::to_string(slot); }

static DcBufs dc_bufs(Context &c, int n, int slot) {
    DcBufs b;
    const size_t nn = (size_t)n * n;
    auto nm = [&](const char *x) { return slot_name(x, slot); };
    b.QA = wsget<double>(c, nm("dc.QA"), nn);
    b.QB = wsget<double>(c, nm("dc.QB"), nn);
    b.U = wsget<double>(c, nm("dc.U"), nn);
    b.lamA = wsget<double>(c, nm("dc.lamA"), n);
    b.lamB = wsget<double>(c, nm("dc.lamB"), n);
    b.dK = wsget<double>(c, nm("dc.dK"), n);
    b.zK = wsget<double>(c, nm("dc.zK"), n);
    b.dv = wsget<double>(c, nm("dc.dv"), n);
    b.Kl = wsget<int>(c, nm("dc.Kl"), n);
    b.defl = wsget<int>(c, nm("dc.defl"), n);
    b.rp = wsget<int>(c, nm("dc.rp"), n);
    b.rn = wsget<int>(c, nm("dc.rn"), n);
    b.rc = wsget<double>(c, nm("dc.rc"), n);
    b.rs = wsget<double>(c, nm("dc.rs"), n);
    b.ord = wsget<int>(c, nm("dc.ord"), n);
    b.tau = wsget<double>(c, nm("dc.tau"), n);
    b.lamK = wsget<double>(c, nm("dc.lamK"), n);
    b.zh = wsget<double>(c, nm("dc.zh"), n);
    b.outc = wsget<int>(c, nm("dc.outc"), n);
    b.kcnt = wsget<int>(c, nm("dc.kcnt"), n);
    b.ndef = wsget<int>(c, nm("dc.ndef"), n);
    b.nrot = wsget<int>(c, nm("dc.nrot"), n);
    b.rho = wsget<double>(c, nm("dc.rho"), n);
    b.status = wsget<int>(c, nm("dc.status"), 1);
    return b;
}

// Eigenvalues (ascending, into w) and eigenvectors (n x n, ld n, returned) of the
// symmetric tridiagonal (d, e).  d and e are device arrays; e has n-1 entries.
static const double *tridiag_dc(Context &c, int n, const double *d, const double *e, double *w, int slot) {
    if (n > kDcMaxN)
        throw Error{DCG_E_ARG, "eigensolver dimension " + std::to_string(n) + " exceeds " + std::to_string(kDcMaxN)};
    DcBufs b = dc_bufs(c, n, slot);
    // Both buffers start at zero: a merge reads whole columns of its node block, including the
    // cross blocks between its two children, which no earlier level writes.
    DCG_CUDA(cudaMemsetAsync(b.QA, 0, sizeof(double) * (size_t)n * n, c.stream));
    DCG_CUDA(cudaMemsetAsync(b.QB, 0, sizeof(double) * (size_t)n * n, c.stream));
    DCG_CUDA(cudaMemsetAsync(b.status, 0, sizeof(int), c.stream));
    dc_leaf_kernel<<<grid1d(n, 256), 256, 0, c.stream>>>(n, d, e, b.lamA, b.QA);
    DCG_LAUNCHED(c);
    DCG_CUDA(cudaFuncSetAttribute(dc_prep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 20 * kDcMaxN));
    for (int half = 1; half < n; half *= 2) {
        const int full = 2 * half;
        const int nodes = (n + full - 1) / full;
        const int nmax = std::min(full, n);
        dc_prep_kernel<<<nodes, 256, 20 * (size_t)nmax, c.stream>>>(n, half, full, e, b);
        DCG_LAUNCHED(c);
        // one warp per root in blocks of two warps: a 792-root merge spreads over 396 blocks,
        // every SM (eight warps a block left 53 of 152 SMs idle on an FP64-bound kernel)
        dc_secular_kernel<<<grid1d((int64_t)n * 32, 64), 64, 0, c.stream>>>(n, full, b);
        DCG_LAUNCHED(c);
        dc_zhat_kernel<<<grid1d((int64_t)n * 32, 64), 64, 0, c.stream>>>(n, full, b);
        DCG_LAUNCHED(c);
        dc_rank_kernel<<<grid1d((int64_t)n * 32, 64), 64, 0, c.stream>>>(n, full, b);
        DCG_LAUNCHED(c);
        dc_vec_kernel<<<n, 128, 0, c.stream>>>(n, full, b);
        DCG_LAUNCHED(c);
        dim3 gg(grid1d(nmax, DG_T), grid1d(nmax, DG_T), nodes);
        dc_gemm_kernel<<<gg, 256, 0, c.stream>>>(n, full, b);
        DCG_LAUNCHED(c);
        std::swap(b.QA, b.QB);
        std::swap(b.lamA, b.lamB);
    }
    DCG_CUDA(cudaMemcpyAsync(w, b.lamA, sizeof(double) * n, cudaMemcpyDeviceToDevice, c.stream));
    // record which buffer holds the result for the vector stage of this slot
    c.eig_Q[slot] = b.QA;
    c.eig_n[slot] = n;
    c.eig_status[slot] = b.status;
    return b.QA;
}

// ===================================================================== 3. back-transformation
// Z = H_0 H_1 ... H_{n-2} Qt(:, vlo:vhi), applied in panels of WY_NB reflectors: the product
// of a panel H_k0 ... H_{k0+nb-1} is I - V T V^H with T upper triangular (the compact WY form
// of Schreiber & Van Loan, SIAM J. Sci. Stat. Comput. 10 (1989) 53), built by the forward
// recurrence T(0:i, i) = -tau_i T(0:i, 0:i) (V(:, 0:i)^H v_i).  Each panel costs three GEMMs.
constexpr int WY_NB = 64;

__global__ void z_from_real_kernel(int n, const double *__restrict__ Qt, int vlo, int nvec, cplx *Z, int64_t ldz) {
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * nvec) return;
    const int i = (int)(idx % n), c = (int)(idx / n);
    Z[i + (int64_t)c * ldz] = mk(Qt[i + (int64_t)(vlo + c) * n], 0.0);
}

// Panel reflectors k0..k0+nbp-1 as a dense (m0 x nbp) matrix, m0 = n-k0-1, row r = global
// row k0+1+r: zero above each reflector's unit entry.
__global__ void wy_extract_kernel(int n, int k0, int nbp, const cplx *__restrict__ A, int64_t lda, cplx *Vp) {
    const int m0 = n - k0 - 1;
    const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (idx >= (int64_t)m0 * nbp) return;
    const int r = (int)(idx % m0), jj = (int)(idx / m0);
    cplx v = mk(0.0, 0.0);
    if (r == jj) v = mk(1.0, 0.0);
    else if (r > jj) v = A[(k0 + 1 + r) + (int64_t)(k0 + jj) * lda];
    Vp[r + (int64_t)jj * m0] = v;
}

// T (nbp x nbp, ld WY_NB) from G = Vp^H Vp and tau[k0..]; one block of WY_NB threads with
// G and T staged in shared memory (the recurrence is sequential in i).
__global__ void wy_tfactor_kernel(int nbp, const cplx *__restrict__ G, const cplx *__restrict__ tau, int k0, cplx *T) {
    extern __shared__ cplx wy_sm[];
    cplx *Gs = wy_sm, *Ts = wy_sm + WY_NB * WY_NB;
    const int j = threadIdx.x;
    for (int x = j; x < WY_NB * WY_NB; x += blockDim.x) {
        Ts[x] = mk(0.0, 0.0);
        const int r = x % WY_NB, cc = x / WY_NB;
        Gs[x] = (r < nbp && cc < nbp) ? G[r + cc * nbp] : mk(0.0, 0.0);
    }
    __syncthreads();
    for (int i = 0; i < nbp; i++) {
        const cplx ti = tau[k0 + i];
        cplx acc = mk(0.0, 0.0);
        if (j < i)
            for (int l = j; l < i; l++) cfma(acc, Ts[j + l * WY_NB], Gs[l + i * WY_NB]);
        __syncthreads();
        if (j < i) Ts[j + i * WY_NB] = cmul(mk(-ti.x, -ti.y), acc);
        if (j == i) Ts[i + i * WY_NB] = ti;
        __syncthreads();
    }
    for (int x = j; x < WY_NB * WY_NB; x += blockDim.x) T[x] = Ts[x];
}

// Register-resident back-transformation (n <= 32 R WPC): WPC warps per eigenvector column,
// the column held in registers (warp w, lane l owns rows l + 32 (WPC i + w)), the reflectors
// applied from the last to the first.  Reflector k-1 is loaded into registers while reflector
// k is applied, so the per-reflector chain is FMAs and shuffles only; this matters most for a
// single column (a CASCI root: n-1 strictly sequential reflections).  With two warps per
// column their partial dot products meet in double-buffered shared memory, summed in a fixed
// order.  Columns are independent, and the FP64 work (8 FMAs per row and reflector) spreads
// over every SM.
template <int R, int WPC, bool PF>
__global__ void __launch_bounds__(64) backtransform_reg_kernel(int n, const cplx *__restrict__ A, int64_t lda,
                                                                const cplx *__restrict__ tau,
                                                                const double *__restrict__ Qt, int vlo, int nvec,
                                                                cplx *Z, int64_t ldz) {
    __shared__ double part[2][2][2];   // [parity][warp][re, im]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wsub = warp % WPC;                               // warp within its column
    const int col = blockIdx.x * (2 / WPC) + warp / WPC;       // 64 threads: 2 / WPC columns
    const bool have = col < nvec;
    cplx z[R], vc[PF ? R : 1], vn[PF ? R : 1];
#pragma unroll
    for (int i = 0; i < R; i++) {
        const int r = lane + 32 * (WPC * i + wsub);
        z[i] = (have && r < n) ? mk(Qt[r + (int64_t)(vlo + col) * n], 0.0) : mk(0.0, 0.0);
    }
#define BT_LOAD(kk, dst)                                                                     \
    {                                                                                        \
        const cplx *v_ = A + (int64_t)(kk) * lda;                                            \
        _Pragma("unroll") for (int i = 0; i < R; i++) {                                      \
            const int r = lane + 32 * (WPC * i + wsub);                                      \
            dst[i] = (have && r > (kk) && r < n) ? __ldg(v_ + r) : mk(0.0, 0.0);             \
        }                                                                                    \
    }
    if (PF && n >= 2) BT_LOAD(n - 2, vc);
    for (int k = n - 2; k >= 0; k--) {
        if (PF && k >= 1) BT_LOAD(k - 1, vn);
        const cplx t = __ldg(tau + k);
        if (t.x != 0.0 || t.y != 0.0) {   // uniform over the block
            const int i0 = (k + 1) / (32 * WPC);   // row chunks below k+1 hold v = 0 in every lane
            double s0r = 0.0, s0i = 0.0, s1r = 0.0, s1i = 0.0;
            const cplx *vk = A + (int64_t)k * lda;
#pragma unroll
            for (int i = 0; i < R; i++) {
                if (i < i0) continue;
                cplx vv;
                if (PF) {
                    vv = vc[i];
                } else {   // read from L1/L2 (shared by the SM's warps) instead of holding it
                    const int r = lane + 32 * (WPC * i + wsub);
                    vv = (have && r > k && r < n) ? __ldg(vk + r) : mk(0.0, 0.0);
                }
                if (i & 1) {   // conj(v) z, two accumulator chains
                    s1r = fma(vv.x, z[i].x, s1r);
                    s1r = fma(vv.y, z[i].y, s1r);
                    s1i = fma(vv.x, z[i].y, s1i);
                    s1i = fma(-vv.y, z[i].x, s1i);
                } else {
                    s0r = fma(vv.x, z[i].x, s0r);
                    s0r = fma(vv.y, z[i].y, s0r);
                    s0i = fma(vv.x, z[i].y, s0i);
                    s0i = fma(-vv.y, z[i].x, s0i);
                }
            }
            double sr = s0r + s1r, si = s0i + s1i;
            for (int o = 16; o > 0; o >>= 1) {
                sr += __shfl_down_sync(0xffffffffu, sr, o);
                si += __shfl_down_sync(0xffffffffu, si, o);
            }
            if (WPC == 2) {
                if (lane == 0) {
                    part[k & 1][wsub][0] = sr;
                    part[k & 1][wsub][1] = si;
                }
                __syncthreads();
                sr = part[k & 1][0][0] + part[k & 1][1][0];
                si = part[k & 1][0][1] + part[k & 1][1][1];
            } else {
                sr = __shfl_sync(0xffffffffu, sr, 0);
                si = __shfl_sync(0xffffffffu, si, 0);
            }
            const double fr = t.x * sr - t.y * si, fi = t.x * si + t.y * sr;   // f = tau (v^H z)
#pragma unroll
            for (int i = 0; i < R; i++) {
                if (i < i0) continue;
                cplx vv;
                if (PF) {
                    vv = vc[i];
                } else {
                    const int r = lane + 32 * (WPC * i + wsub);
                    vv = (have && r > k && r < n) ? __ldg(vk + r) : mk(0.0, 0.0);
                }
                z[i].x = fma(-vv.x, fr, z[i].x);   // z -= v f
                z[i].x = fma(vv.y, fi, z[i].x);
                z[i].y = fma(-vv.x, fi, z[i].y);
                z[i].y = fma(-vv.y, fr, z[i].y);
            }
        }
        if (PF) {
#pragma unroll
            for (int i = 0; i < R; i++) vc[i] = vn[i];
        }
    }
#undef BT_LOAD
    if (have) {
#pragma unroll
        for (int i = 0; i < R; i++) {
            const int r = lane + 32 * (WPC * i + wsub);
            if (r < n) Z[r + (int64_t)col * ldz] = z[i];
        }
    }
}

template <int R, int WPC, bool PF>
static void launch_bt_reg(Context &c, int n, const cplx *A, int64_t lda, const cplx *tau, const double *Qt, int vlo,
                          int nvec, cplx *Z, int64_t ldz) {
    backtransform_reg_kernel<R, WPC, PF><<<grid1d(nvec, 2 / WPC), 64, 0, c.stream>>>(n, A, lda, tau, Qt, vlo, nvec,
                                                                                       Z, ldz);
    DCG_LAUNCHED(c);
}

// ===================================================================== driver
struct HeevWork {
    double *d, *e;
    cplx *tau, *ppart, *w;
};

static HeevWork heev_work(Context &c, int n, int slot) {
    HeevWork h;
    h.d = wsget<double>(c, slot_name("heev.d", slot), n + 1);
    h.e = wsget<double>(c, slot_name("heev.e", slot), n + 1);
    h.tau = wsget<cplx>(c, slot_name("heev.tau", slot), n + 1);
    int nchunk = (n + HH_CHUNK - 1) / HH_CHUNK;
    h.ppart = wsget<cplx>(c, slot_name("heev.ppart", slot), (size_t)nchunk * (n + 1));
    h.w = wsget<cplx>(c, slot_name("heev.w", slot), n + 1);
    return h;
}

// Cooperative launches from different contexts (a serving process runs one context per
// slot, each on its own stream) are serialised from launch to completion: two grid-synchronised
// kernels must never wait for each other's SMs.
static std::mutex g_coop_mutex;

// A fresh barrier (counters and error flag zero) with the context's wait limit, written in
// stream order (a copy from pageable host memory is staged before the call returns).
static void gridbar_reset(Context &c, GridBar *gb) {
    GridBar x{};
    x.limit_ns = c.wait_limit_ns ? c.wait_limit_ns : kBarrierLimitNs;
    DCG_CUDA(cudaMemcpyAsync(gb, &x, sizeof(GridBar), cudaMemcpyHostToDevice, c.stream));
}

static void tridiag_persistent(Context &c, int n, cplx *A, int64_t lda, HeevWork &h) {
    std::lock_guard<std::mutex> coop(g_coop_mutex);
    const size_t smem = 2 * sizeof(cplx) * (size_t)std::max(n - 1, 1);
    DCG_CUDA(cudaFuncSetAttribute(tridiag_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int per_sm = 0;
    DCG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tridiag_persistent_kernel, TRD_THREADS, smem));
    if (per_sm < 1) throw Error{DCG_E_CUDA, "tridiagonalisation kernel does not fit on an SM"};
    // one warp per trailing column at most; never more blocks than can be co-resident
    const int want = std::max(1, (n + (TRD_THREADS / 32) - 1) / (TRD_THREADS / 32));
    const int nblocks = std::min({want, per_sm * std::max(1, c.num_sms), 2 * std::max(1, c.num_sms)});
    cplx *pbuf = wsget<cplx>(c, "trd.p", (size_t)n + 1);
    double2 *part = wsget<double2>(c, "trd.part", (size_t)nblocks + 1);
    GridBar *gb = wsget<GridBar>(c, "trd.bar", 1);
    gridbar_reset(c, gb);
    void *args[] = {&n, &A, &lda, &h.d, &h.e, &h.tau, &pbuf, &part, &gb};
    DCG_CUDA(cudaLaunchCooperativeKernel((const void *)tridiag_persistent_kernel, dim3(nblocks), dim3(TRD_THREADS),
                                         args, smem, c.stream));
    DCG_LAUNCHED(c);
    GridBar hb;
    DCG_CUDA(cudaMemcpyAsync(&hb, gb, sizeof(GridBar), cudaMemcpyDeviceToHost, c.stream));
    DCG_CUDA(cudaStreamSynchronize(c.stream));
    if (hb.err) throw Error{DCG_E_NUMERIC, "tridiagonalisation: a grid barrier wait timed out"};
}

// Shared-memory tridiagonalisation of several matrices in one cooperative launch (one job = one
// block group).  Block counts come from a cost model: a job's FP64 work (about 4 n^3 FMAs; a
// GB300 SM retires ~2 FP64 FMAs per clock) spreads over its blocks while the per-column grid barrier
// and reflector wait cost more with more blocks; the jobs share the SMs, and blocks go to the job that
// is currently the slowest.  Returns false (nothing launched) when the jobs do not fit.
static double trd_cost(int n, int nb) {
    return 4.0 * (double)n * n * n / (nb * 4.0e9) + 1.4 * n * (3.0e-6 + 0.02e-6 * nb);   // one barrier + one signal
}

static size_t trd_bytes_for(int n, int nbk) { return (size_t)(((n + nbk - 1) / nbk) + 2) * n * sizeof(cplx); }

// Shared-memory limit of one block of the batched kernel (its static shared memory aside).
static size_t trd_smem_limit(const Context &c) {
    int optin = 0;
    DCG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c.device));
    return (size_t)std::max(0, optin - 1024);
}

// Block groups of one batched launch: every job gets the fewest blocks whose shared memory holds
// its columns, then the remaining SMs go one by one to the job that is currently the slowest
// and that they help (trd_cost); b0 and the largest block's shared memory follow.  False when
// the jobs do not fit one launch.
static bool trd_plan(const Context &c, std::vector<TrdJob> &jobs, int &total, size_t &smem) {
    const int sms = std::max(1, c.num_sms);
    const size_t limit = trd_smem_limit(c);
    total = 0;
    for (TrdJob &j : jobs) {
        if (j.n > kTridiagSmemMaxN) return false;
        int nb = 1;
        while (nb < std::min(sms, j.n) && trd_bytes_for(j.n, nb) > limit) nb++;
        if (trd_bytes_for(j.n, nb) > limit) return false;
        j.nb = nb;
        total += nb;
    }
    if (total > sms) return false;
    while (total < sms) {   // give the next block to the slowest job that it helps
        int best = -1;
        double worst = -1.0;
        for (size_t q = 0; q < jobs.size(); q++) {
            const TrdJob &j = jobs[q];
            if (j.nb >= j.n || trd_cost(j.n, j.nb + 1) >= trd_cost(j.n, j.nb)) continue;
            const double cst = trd_cost(j.n, j.nb);
            if (cst > worst) {
                worst = cst;
                best = (int)q;
            }
        }
        if (best < 0) break;
        jobs[best].nb++;
        total++;
    }
    smem = 0;
    int b0 = 0;
    for (TrdJob &j : jobs) {
        smem = std::max(smem, trd_bytes_for(j.n, j.nb));
        j.b0 = b0;
        b0 += j.nb;
    }
    DCG_CUDA(cudaFuncSetAttribute(tridiag_smem_batched_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit));
    int per_sm = 0;
    DCG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, tridiag_smem_batched_kernel, TRD_THREADS, smem));
    return per_sm >= 1 && total <= per_sm * sms;
}

// The cooperative launch of planned jobs on `stream` (their barriers already reset in stream
// order), then their barrier error flags, read back after the launch completes.
static std::vector<GridBar> trd_launch(Context &c, std::vector<TrdJob> &jobs, int total, size_t smem,
                                       cudaStream_t stream, const char *table) {
    TrdJob *dj = wsget<TrdJob>(c, table, jobs.size());
    DCG_CUDA(cudaMemcpyAsync(dj, jobs.data(), jobs.size() * sizeof(TrdJob), cudaMemcpyHostToDevice, stream));
    int nj = (int)jobs.size();
    void *args[] = {&dj, &nj};
    DCG_CUDA(cudaLaunchCooperativeKernel((const void *)tridiag_smem_batched_kernel, dim3(total), dim3(TRD_THREADS),
                                         args, smem, stream));
    DCG_CUDA(cudaGetLastError());
    std::vector<GridBar> hb(jobs.size());
    for (size_t q = 0; q < jobs.size(); q++)
        DCG_CUDA(cudaMemcpyAsync(&hb[q], jobs[q].gb, sizeof(GridBar), cudaMemcpyDeviceToHost, stream));
    DCG_CUDA(cudaStreamSynchronize(stream));
    return hb;
}

// ---- merging the reductions of several contexts (the serving loop's slots)
// A context with merge_reductions set hands its batched reduction to a per-device batcher
// instead of launching it.  The first waiting thread that finds the batcher idle becomes the
// leader: it takes, in arrival order, the submissions whose jobs fit one launch together, makes
// a batcher stream wait for each submission's ready event, launches them as one cooperative
// kernel (each job its own block group and barrier) and hands every submission its result.
// Requests that run concurrently then overlap their barrier-bound column loops inside one kernel
// instead of queueing on the cooperative-launch lock.  The block-group sizes change with the
// company, the arithmetic of a job does not: its partial sums do not depend on the number of
// blocks reducing it, so a matrix gets the same bits alone and merged.
struct CoopSub {
    Context *c = nullptr;
    std::vector<TrdJob> jobs;
    cudaEvent_t ready = nullptr;
    int state = 0;   // 0 waiting, 1 reduced, 2 does not fit a launch, 3 a wait timed out, 4 CUDA error
    std::string msg;
};

struct CoopBatcher {
    std::mutex mu;
    std::condition_variable cv;
    std::deque<CoopSub *> pending;
    bool busy = false;
    cudaStream_t stream = nullptr;
    int64_t launches = 0, joint = 0, carried = 0;
};

static std::mutex g_batchers_mu;
static std::map<int, CoopBatcher *> g_batchers;   // per device, for the life of the process

static CoopBatcher &coop_batcher(int device) {
    std::lock_guard<std::mutex> lk(g_batchers_mu);
    CoopBatcher *&b = g_batchers[device];
    if (!b) {
        b = new CoopBatcher;
        DCG_CUDA(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
    }
    return *b;
}

// One joint launch of the taken submissions (leader thread, leader context's workspace).
static void coop_run(Context &leader, CoopBatcher &B, std::vector<CoopSub *> &take) {
    std::vector<TrdJob> all;
    for (CoopSub *s : take) all.insert(all.end(), s->jobs.begin(), s->jobs.end());
    try {
        std::lock_guard<std::mutex> coop(g_coop_mutex);
        int total = 0;
        size_t smem = 0;
        if (!trd_plan(leader, all, total, smem)) throw Error{DCG_E_CUDA, "merged reduction does not fit"};
        for (CoopSub *s : take) DCG_CUDA(cudaStreamWaitEvent(B.stream, s->ready, 0));
        const std::vector<GridBar> hb = trd_launch(leader, all, total, smem, B.stream, "trd.jobs.joint");
        size_t q = 0;
        for (CoopSub *s : take) {
            bool err = false;
            for (size_t k = 0; k < s->jobs.size(); k++, q++) err = err || hb[q].err != 0;
            s->state = err ? 3 : 1;
            s->c->launches++;
        }
        B.launches++;
        if (take.size() > 1) B.joint++;
        B.carried += (int64_t)take.size();
    } catch (const Error &e) {
        for (CoopSub *s : take) {
            s->state = 4;
            s->msg = e.msg;
        }
    }
}

static bool tridiag_smem_merged(Context &c, std::vector<TrdJob> &jobs) {
    {   // a submission that cannot run even alone goes the unbatched way
        std::vector<TrdJob> alone = jobs;
        int total = 0;
        size_t smem = 0;
        if (!trd_plan(c, alone, total, smem)) return false;
    }
    for (TrdJob &j : jobs) gridbar_reset(c, j.gb);
    CoopSub me;
    me.c = &c;
    me.jobs = jobs;
    DCG_CUDA(cudaEventCreateWithFlags(&me.ready, cudaEventDisableTiming));
    const cudaError_t er = cudaEventRecord(me.ready, c.stream);
    if (er != cudaSuccess) {
        cudaEventDestroy(me.ready);
        throw Error{DCG_E_CUDA, std::string("cudaEventRecord: ") + cudaGetErrorString(er)};
    }
    CoopBatcher &B = coop_batcher(c.device);
    // merge window: a leader that finds no other submission waits this long for one
    // (DCG_MERGE_WINDOW_US, default 0: launch at once)
    const char *wenv = getenv("DCG_MERGE_WINDOW_US");
    const long window_us = wenv ? std::max(0L, std::min(5000000L, atol(wenv))) : 0L;
    {
        std::unique_lock<std::mutex> lk(B.mu);
        B.pending.push_back(&me);
        B.cv.notify_all();
        while (me.state == 0) {
            if (B.busy) {
                B.cv.wait(lk);
                continue;
            }
            B.busy = true;
            if (window_us > 0 && B.pending.size() < 2)
                B.cv.wait_for(lk, std::chrono::microseconds(window_us), [&] { return B.pending.size() >= 2; });
            std::vector<CoopSub *> take;
            std::vector<TrdJob> trial;
            while (!B.pending.empty()) {
                CoopSub *s = B.pending.front();
                std::vector<TrdJob> t2 = trial;
                t2.insert(t2.end(), s->jobs.begin(), s->jobs.end());
                int total = 0;
                size_t smem = 0;
                bool fits = false;
                try {
                    fits = trd_plan(c, t2, total, smem);
                } catch (const Error &) {
                    fits = false;
                }
                if (!fits && !take.empty()) break;   // the rest waits for the next launch
                B.pending.pop_front();
                if (!fits) {                            // cannot run merged at all
                    s->state = 2;
                    continue;
                }
                take.push_back(s);
                trial.swap(t2);
            }
            lk.unlock();
            if (!take.empty()) coop_run(c, B, take);
            lk.lock();
            B.busy = false;
            B.cv.notify_all();
        }
    }
    cudaEventDestroy(me.ready);
    if (me.state == 2) return false;
    if (me.state == 3) throw Error{DCG_E_NUMERIC, "tridiagonalisation: a grid barrier wait timed out"};
    if (me.state == 4) throw Error{DCG_E_CUDA, "merged tridiagonalisation: " + me.msg};
    return true;
}

// Cluster launch of jobs of order <= kTridiagClusterMaxN that share a cluster shape (ncta
// blocks each): one cluster per job, no grid-wide synchronisation, so no cooperative launch
// and no serialisation against other contexts.  False when no cluster of this shape can be
// resident (the caller then uses the cooperative form).
static bool tridiag_cluster_group(Context &c, std::vector<TrdJob> &jobs, int ncta) {
    size_t smem = 0;
    for (const TrdJob &j : jobs) smem = std::max(smem, trd_cluster_bytes(j.n, ncta));
    const size_t limit = trd_smem_limit(c);
    if (smem > limit) return false;
    // the same values from every context and thread (serving slots launch concurrently), so
    // no launch can see another's smaller limit
    DCG_CUDA(cudaFuncSetAttribute(tridiag_cluster_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit));
    DCG_CUDA(cudaFuncSetAttribute(tridiag_cluster_kernel, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)ncta;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(ncta * jobs.size()));
    cfg.blockDim = dim3(TRD_THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = c.stream;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    int resident = 0;
    if (cudaOccupancyMaxActiveClusters(&resident, (const void *)tridiag_cluster_kernel, &cfg) != cudaSuccess ||
        resident < 1) {
        cudaGetLastError();
        return false;
    }
    for (const TrdJob &j : jobs) gridbar_reset(c, j.gb);
    TrdJob *dj = wsget<TrdJob>(c, "trdc.jobs" + std::to_string(ncta), jobs.size());
    DCG_CUDA(cudaMemcpyAsync(dj, jobs.data(), jobs.size() * sizeof(TrdJob), cudaMemcpyHostToDevice, c.stream));
    int *st = wsget<int>(c, "trdc.status", 1);
    DCG_CUDA(cudaMemsetAsync(st, 0, sizeof(int), c.stream));
    const TrdJob *djc = dj;
    const int nj = (int)jobs.size();
    DCG_CUDA(cudaLaunchKernelEx(&cfg, tridiag_cluster_kernel, djc, nj, ncta, (unsigned)smem, st));
    DCG_LAUNCHED(c);
    std::vector<GridBar> hb(jobs.size());
    for (size_t q = 0; q < jobs.size(); q++)
        DCG_CUDA(cudaMemcpyAsync(&hb[q], jobs[q].gb, sizeof(GridBar), cudaMemcpyDeviceToHost, c.stream));
    int hst = 0;
    DCG_CUDA(cudaMemcpyAsync(&hst, st, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    DCG_CUDA(cudaStreamSynchronize(c.stream));
    if (hst) throw Error{DCG_E_CUDA, "tridiagonalisation: cluster launch shape check " + std::to_string(hst)};
    for (const GridBar &g : hb)
        if (g.err) throw Error{DCG_E_NUMERIC, "tridiagonalisation: a cluster wait timed out"};
    return true;
}

// Whether the cluster form takes the matrices it fits (DCG_TRD_CLUSTER=1).  Off by default:
// on GB300 it measured slower than the cooperative form (the 300 x 300 Fock block 6.4 ms on
// 16 SMs against 4.35 ms on 63, the B-G batch 1.84 against 1.73 ms): a 16-block cluster
// carries four times the per-block FP64 work of a column, more than its faster exchange saves.
static bool trd_cluster_enabled() {
    static const bool on = [] {
        const char *e = getenv("DCG_TRD_CLUSTER");
        return e && e[0] == '1';
    }();
    return on;
}

static bool tridiag_smem_batched(Context &c, std::vector<TrdJob> &jobs) {
    if (c.merge_reductions) return tridiag_smem_merged(c, jobs);
    std::lock_guard<std::mutex> coop(g_coop_mutex);
    int total = 0;
    size_t smem = 0;
    if (!trd_plan(c, jobs, total, smem)) return false;
    for (size_t q = 0; q < jobs.size(); q++) gridbar_reset(c, jobs[q].gb);
    const std::vector<GridBar> hb = trd_launch(c, jobs, total, smem, c.stream, "trd.jobs");
    c.launches++;
    for (const GridBar &g : hb)
        if (g.err) throw Error{DCG_E_NUMERIC, "tridiagonalisation: a grid barrier wait timed out"};
    return true;
}

// One matrix: the L2-resident persistent kernel, or one kernel launch per column beyond it.
static void tridiag_single(Context &c, int n, cplx *A, int64_t lda, HeevWork &h) {
    if (n <= kTridiagPersistentMaxN) {
        tridiag_persistent(c, n, A, lda, h);
        return;
    }
    for (int k = 0; k + 1 < n; k++) {
        const int m = n - k - 1;
        hh_gen_kernel<<<1, 256, 0, c.stream>>>(n, k, A, lda, h.d, h.e, h.tau);
        DCG_LAUNCHED(c);
        const int nchunk = (m + HH_CHUNK - 1) / HH_CHUNK;
        dim3 g1(grid1d(m, 128), nchunk);
        hh_matvec_kernel<<<g1, 128, 0, c.stream>>>(n, k, A, lda, h.tau, h.ppart);
        DCG_LAUNCHED(c);
        hh_w_kernel<<<1, 512, 0, c.stream>>>(n, k, A, lda, h.tau, h.ppart, nchunk, h.w);
        DCG_LAUNCHED(c);
        dim3 g2(grid1d(m, 128), m);
        hh_update_kernel<<<g2, 128, 0, c.stream>>>(n, k, A, lda, h.w);
        DCG_LAUNCHED(c);
    }
    hh_last_kernel<<<1, 1, 0, c.stream>>>(n, A, lda, h.d);
    DCG_LAUNCHED(c);
}

static void check_dc_status(Context &c, int slot) {
    if (!c.eig_status[slot]) return;
    int st = 0;
    DCG_CUDA(cudaMemcpyAsync(&st, c.eig_status[slot], sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    DCG_CUDA(cudaStreamSynchronize(c.stream));
    if (st) throw Error{DCG_E_NUMERIC, "divide-and-conquer merge met coincident undeflated poles"};
}

// Eigenvalues of every job's matrix (ascending, into job.w); the reflectors stay in job.A and
// the tridiagonal eigenvectors in the job's slot for heev_vectors_slot.  Jobs that fit the
// shared-memory tridiagonalisation are reduced together in one launch.
void heev_values_batched(Context &c, const std::vector<EigJob> &jobs) {
    if (jobs.empty()) return;
    double work = 0.0;
    for (const EigJob &j : jobs) {
        if (j.slot < 0 || j.slot >= kEigSlots) throw Error{DCG_E_ARG, "eigensolver slot out of range"};
        work += (16.0 / 3.0) * (double)j.n * j.n * j.n;
    }
    std::vector<HeevWork> hw;
    for (const EigJob &j : jobs) hw.push_back(heev_work(c, std::max(j.n, 1), j.slot));
    FamScope fs(c, DCG_FAM_EIG, work);
    {
        FamScope f1(c, DCG_FAM_EIG_TRI, work);
        std::vector<TrdJob> tj;
        std::vector<size_t> who;
        for (size_t q = 0; q < jobs.size(); q++) {
            const EigJob &j = jobs[q];
            if (j.n <= 0 || j.n > kTridiagSmemMaxN) continue;
            TrdJob t;
            t.A = j.A;
            t.lda = j.lda;
            t.d = hw[q].d;
            t.e = hw[q].e;
            t.tau = hw[q].tau;
            t.pbuf = wsget<cplx>(c, slot_name("trd.p", j.slot), 2 * ((size_t)j.n + 1));   // two parities
            t.part = wsget<double2>(c, slot_name("trd.part", j.slot), 2 * ((size_t)j.n + 1));   // two parities
            t.gb = wsget<GridBar>(c, slot_name("trd.bar", j.slot), 1);
            t.n = j.n;
            t.b0 = t.nb = 0;
            tj.push_back(t);
            who.push_back(q);
        }
        std::vector<bool> done(jobs.size(), false);
        if (!tj.empty() && trd_cluster_enabled()) {   // small matrices: one cluster each
            std::map<int, std::vector<size_t>> groups;   // blocks per cluster -> indices into tj
            for (size_t k = 0; k < tj.size(); k++)
                if (tj[k].n <= kTridiagClusterMaxN) groups[trd_cluster_ctas(tj[k].n)].push_back(k);
            std::vector<bool> taken(tj.size(), false);
            for (auto &g : groups) {
                std::vector<TrdJob> gj;
                for (size_t k : g.second) gj.push_back(tj[k]);
                if (!tridiag_cluster_group(c, gj, g.first)) continue;
                for (size_t k : g.second) {
                    taken[k] = true;
                    done[who[k]] = true;
                }
            }
            std::vector<TrdJob> rest;
            std::vector<size_t> rwho;
            for (size_t k = 0; k < tj.size(); k++)
                if (!taken[k]) {
                    rest.push_back(tj[k]);
                    rwho.push_back(who[k]);
                }
            tj.swap(rest);
            who.swap(rwho);
        }
        if (!tj.empty()) {
            if (tridiag_smem_batched(c, tj)) {
                for (size_t q : who) done[q] = true;
            } else if (tj.size() > 1) {   // too many for one launch: each on its own
                for (size_t k = 0; k < tj.size(); k++) {
                    std::vector<TrdJob> one(1, tj[k]);
                    if (tridiag_smem_batched(c, one)) done[who[k]] = true;
                }
            }
        }
        for (size_t q = 0; q < jobs.size(); q++)
            if (!done[q] && jobs[q].n > 0) tridiag_single(c, jobs[q].n, jobs[q].A, jobs[q].lda, hw[q]);
    }
    {
        FamScope f2(c, DCG_FAM_EIG_VAL, work / 4.0);
        std::vector<size_t> dq;   // largest first, so the long chains start first
        for (size_t q = 0; q < jobs.size(); q++)
            if (jobs[q].n > 0 && !jobs[q].tridiag_only) dq.push_back(q);
        std::stable_sort(dq.begin(), dq.end(), [&](size_t x, size_t y) { return jobs[x].n > jobs[y].n; });
        on_aux_streams(c, (int)dq.size(), [&](int k) {
            const size_t q = dq[k];
            tridiag_dc(c, jobs[q].n, hw[q].d, hw[q].e, jobs[q].w, jobs[q].slot);
        });
    }
    for (const EigJob &j : jobs)
        if (j.n > 0 && !j.tridiag_only) check_dc_status(c, j.slot);
}

// y <- Q^H y for the columns of Y0 (written to Y), Q = H_0 H_1 ... H_{n-2} the reflectors of a
// tridiagonal reduction (H_k = I - tau_k v_k v_k^H, v_k in column k of A below the diagonal):
// H_0^H first.  One warp per column, the column in registers (R = ceil(n / 32)).
template <int R, int WPC>
__global__ void __launch_bounds__(64) apply_qh_kernel(int n, const cplx *__restrict__ A, int64_t lda,
                                                     const cplx *__restrict__ tau, const cplx *__restrict__ Y0,
                                                     int64_t ldy0, int ncol, cplx *Y, int64_t ldy) {
    __shared__ double part[2][2][2];   // [parity][warp][re, im]
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wsub = warp % WPC;                              // warp within its column
    const int col = blockIdx.x * (2 / WPC) + warp / WPC;      // 64 threads: 2 / WPC columns
    const bool have = col < ncol;
    if (WPC == 1 && !have) return;   // whole warp; with two warps per column both stay for the barriers
    cplx z[R];
#pragma unroll
    for (int i = 0; i < R; i++) {
        const int r = lane + 32 * (WPC * i + wsub);
        z[i] = (have && r < n) ? Y0[r + (int64_t)col * ldy0] : mk(0.0, 0.0);
    }
    for (int k = 0; k + 1 < n; k++) {
        const cplx t = __ldg(tau + k);
        if (t.x == 0.0 && t.y == 0.0) continue;   // uniform over the block
        const int i0 = (k + 1) / (32 * WPC);      // row chunks below k+1 hold v = 0 in every lane
        const cplx *vk = A + (int64_t)k * lda;
        double sr = 0.0, si = 0.0;
#pragma unroll
        for (int i = 0; i < R; i++) {
            if (i < i0) continue;
            const int r = lane + 32 * (WPC * i + wsub);
            const cplx vv = (have && r > k && r < n) ? __ldg(vk + r) : mk(0.0, 0.0);
            sr = fma(vv.x, z[i].x, fma(vv.y, z[i].y, sr));    // conj(v) z
            si = fma(vv.x, z[i].y, fma(-vv.y, z[i].x, si));
        }
        for (int o = 16; o > 0; o >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, o);
            si += __shfl_xor_sync(0xffffffffu, si, o);
        }
        if (WPC == 2) {   // the two warps' partial dots, summed in a fixed order
            if (lane == 0) {
                part[k & 1][wsub][0] = sr;
                part[k & 1][wsub][1] = si;
            }
            __syncthreads();
            sr = part[k & 1][0][0] + part[k & 1][1][0];
            si = part[k & 1][0][1] + part[k & 1][1][1];
        }
        const double fr = t.x * sr + t.y * si, fi = t.x * si - t.y * sr;   // f = conj(tau) (v^H z)
#pragma unroll
        for (int i = 0; i < R; i++) {
            if (i < i0) continue;
            const int r = lane + 32 * (WPC * i + wsub);
            const cplx vv = (have && r > k && r < n) ? __ldg(vk + r) : mk(0.0, 0.0);
            z[i].x = fma(-vv.x, fr, fma(vv.y, fi, z[i].x));   // z -= v f
            z[i].y = fma(-vv.x, fi, fma(-vv.y, fr, z[i].y));
        }
    }
    if (!have) return;
#pragma unroll
    for (int i = 0; i < R; i++) {
        const int r = lane + 32 * (WPC * i + wsub);
        if (r < n) Y[r + (int64_t)col * ldy] = z[i];
    }
}

// Per outer index o (one thread): solve (T + alpha_o) z = y_o by Gaussian elimination with
// partial pivoting on the tridiagonal (Golub & Van Loan, Matrix Computations, 4th ed., 4.3:
// row interchanges add one superdiagonal of fill-in), then e2o = -Re y^H z, sco = |z|^2.
// T: diagonal d (n), off-diagonal e (n-1), real.  The eliminated rows go to per-thread scratch
// laid out [row * nouter + o] (coalesced across threads).
__global__ void tridiag_solve_e2_kernel(int n, const double *__restrict__ d, const double *__restrict__ e,
                                        const cplx *__restrict__ Y, int64_t ldy, int nouter,
                                        const double *__restrict__ alpha, double *D, double *U, double *U2, cplx *B,
                                        double *e2o, double *sco) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nouter) return;
    const double al = alpha[o];
    const cplx *y = Y + (int64_t)o * ldy;
#define IX(k) ((int64_t)(k) * nouter + o)
    double dcur = d[0] + al, ucur = n > 1 ? e[0] : 0.0;
    cplx bcur = y[0];
    for (int i = 0; i + 1 < n; i++) {
        double dn = d[i + 1] + al;
        double un = (i + 2 < n) ? e[i + 1] : 0.0;
        cplx bn = y[i + 1];
        const double dl = e[i];
        double u2 = 0.0;
        if (fabs(dcur) >= fabs(dl)) {   // pivot on row i
            const double f = dl / dcur;
            dn = fma(-f, ucur, dn);
            bn = mk(fma(-f, bcur.x, bn.x), fma(-f, bcur.y, bn.y));
        } else {                        // rows i and i+1 exchanged
            const double f = dcur / dl;
            const double newu = dn;
            dn = fma(-f, dn, ucur);
            u2 = un;
            un = -f * un;
            const cplx nb = mk(fma(-f, bn.x, bcur.x), fma(-f, bn.y, bcur.y));
            bcur = bn;
            bn = nb;
            dcur = dl;
            ucur = newu;
        }
        D[IX(i)] = dcur;
        U[IX(i)] = ucur;
        U2[IX(i)] = u2;
        B[IX(i)] = bcur;
        dcur = dn;
        ucur = un;
        bcur = bn;
    }
    // back substitution, with the two sums
    double er = 0.0, s = 0.0;
    cplx z1 = mk(bcur.x / dcur, bcur.y / dcur), z2 = mk(0.0, 0.0);
    er += y[n - 1].x * z1.x + y[n - 1].y * z1.y;
    s += z1.x * z1.x + z1.y * z1.y;
    for (int i = n - 2; i >= 0; i--) {
        const double di = D[IX(i)], ui = U[IX(i)], u2i = U2[IX(i)];
        const cplx bi = B[IX(i)];
        const cplx zi = mk((bi.x - ui * z1.x - u2i * z2.x) / di, (bi.y - ui * z1.y - u2i * z2.y) / di);
        er += y[i].x * zi.x + y[i].y * zi.y;
        s += zi.x * zi.x + zi.y * zi.y;
        z2 = z1;
        z1 = zi;
    }
#undef IX
    e2o[o] = -er;
    sco[o] = s;
}

void tridiag_e2(Context &c, int slot, int n, const cplx *A, int64_t lda, const cplx *VC, int64_t ldvc, int nouter,
                const double *alpha, double *e2o, double *sco) {
    if (n <= 0 || nouter <= 0) return;
    if (n > kTridiagE2MaxN) throw Error{DCG_E_ARG, "tridiag_e2: dimension above the register limit"};
    HeevWork h = heev_work(c, n, slot);
    cplx *Y = wsget<cplx>(c, slot_name("te2.Y", slot), (size_t)n * nouter);
    FamScope fs(c, DCG_FAM_EIG, 8.0 * (double)n * n * nouter);
    // one warp per vector up to 256 rows; above, two warps per vector (twice the warps to hide
    // the per-reflector reduction latency) and the register chunks sized to the rows
    if (n <= 256) {
        apply_qh_kernel<8, 1><<<grid1d(nouter, 2), 64, 0, c.stream>>>(n, A, lda, h.tau, VC, ldvc, nouter, Y, n);
    } else {
        const unsigned g = (unsigned)nouter;
        if (n <= 512) apply_qh_kernel<8, 2><<<g, 64, 0, c.stream>>>(n, A, lda, h.tau, VC, ldvc, nouter, Y, n);
        else if (n <= 768) apply_qh_kernel<12, 2><<<g, 64, 0, c.stream>>>(n, A, lda, h.tau, VC, ldvc, nouter, Y, n);
        else if (n <= 896) apply_qh_kernel<14, 2><<<g, 64, 0, c.stream>>>(n, A, lda, h.tau, VC, ldvc, nouter, Y, n);
        else apply_qh_kernel<16, 2><<<g, 64, 0, c.stream>>>(n, A, lda, h.tau, VC, ldvc, nouter, Y, n);
    }
    DCG_LAUNCHED(c);
    const size_t sz = (size_t)n * nouter;
    double *D = wsget<double>(c, slot_name("te2.D", slot), sz);
    double *U = wsget<double>(c, slot_name("te2.U", slot), sz);
    double *U2 = wsget<double>(c, slot_name("te2.U2", slot), sz);
    cplx *B = wsget<cplx>(c, slot_name("te2.B", slot), sz);
    // one thread per outer index, its tridiagonal solve a serial FP64 chain: blocks of one warp
    // spread the indices over as many SMs as there are warps
    tridiag_solve_e2_kernel<<<grid1d(nouter, 32), 32, 0, c.stream>>>(n, h.d, h.e, Y, n, nouter, alpha, D, U, U2, B,
                                                                      e2o, sco);
    DCG_LAUNCHED(c);
}

// Eigenvectors [vlo, vhi) of the matrix reduced in slot `slot` by heev_values_batched (its
// reflectors still in A, its tridiagonal eigenvectors in the slot).
void heev_vectors_slot(Context &c, int slot, int n, cplx *A, int64_t lda, int vlo, int vhi, cplx *Z, int64_t ldz) {
    const int nvec = vhi - vlo;
    if (nvec <= 0 || n <= 0 || Z == nullptr) return;
    if (slot < 0 || slot >= kEigSlots || c.eig_Q[slot] == nullptr || c.eig_n[slot] != n)
        throw Error{DCG_E_STATE, "eigenvectors requested without a matching eigenvalue stage"};
    HeevWork h = heev_work(c, n, slot);
    const double *Qt = c.eig_Q[slot];
    FamScope fs(c, DCG_FAM_EIG, 8.0 * (double)n * n * nvec);
    FamScope f4(c, DCG_FAM_EIG_BACK, 8.0 * (double)n * n * nvec);
    // Many columns: the FP64 pipe is the limit, one warp per column without prefetch (fewest
    // registers).  Few columns: the n-1 sequential reflections are the limit, prefetch the next
    // reflector (two warps per column above 512 rows to keep it in registers).
    if (n <= 1024) {
        const bool many = nvec >= 64;
        if (n <= 256) {
            if (many) launch_bt_reg<8, 1, false>(c, n, A, lda, h.tau, Qt, vlo, nvec, Z, ldz);
            else launch_bt_reg<8, 1, true>(c, n, A, lda, h.tau, Qt, vlo, nvec, Z, ldz);
        } else if (n <= 512) {
            if (many) launch_bt_reg<8, 2, false>(c, n, A, lda, h.tau, Qt, vlo, nvec, Z, ldz);
            else launch_bt_reg<16, 1, true>(c, n, A, lda, h.tau, Qt, vlo, nvec, Z, ldz);
        } else {
            // many columns: two warps per column, register chunks sized to the rows (a 792-row
            // column in 14 chunks instead of 32 one-warp chunks of which 7 are empty)
            if (many) {
                if (n <= 768) launch_bt_reg<12, 2, false>(c, n, A, lda, h.tau, Qt, vlo, nvec, Z, ldz);
                else if (n <= 896) launch_bt_reg<14, 2, false>(c, n, A, lda, h.tau, Qt, vlo, nvec, Z, ldz);
                else launch_bt_reg<16, 2, false>(c, n, A, lda, h.tau, Qt, vlo, nvec, Z, ldz);
            } else {
                launch_bt_reg<16, 2, true>(c, n, A, lda, h.tau, Qt, vlo, nvec, Z, ldz);
            }
        }
        return;
    }
    z_from_real_kernel<<<grid1d((int64_t)n * nvec, 256), 256, 0, c.stream>>>(n, Qt, vlo, nvec, Z, ldz);
    DCG_LAUNCHED(c);
    cplx *Vp = wsget<cplx>(c, "wy.V", (size_t)n * WY_NB);
    cplx *G = wsget<cplx>(c, "wy.G", WY_NB * WY_NB);
    cplx *T = wsget<cplx>(c, "wy.T", WY_NB * WY_NB);
    cplx *W1 = wsget<cplx>(c, "wy.W1", (size_t)WY_NB * nvec);
    cplx *W2 = wsget<cplx>(c, "wy.W2", (size_t)WY_NB * nvec);
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0), mone = mk(-1.0, 0.0);
    const int nref = n - 1;
    const int npanel = (nref + WY_NB - 1) / WY_NB;
    DCG_CUDA(cudaFuncSetAttribute(wy_tfactor_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  2 * WY_NB * WY_NB * (int)sizeof(cplx)));
    for (int p = npanel - 1; p >= 0; p--) {
        const int k0 = p * WY_NB;
        const int nbp = std::min(WY_NB, nref - k0);
        const int m0 = n - k0 - 1;
        wy_extract_kernel<<<grid1d((int64_t)m0 * nbp, 256), 256, 0, c.stream>>>(n, k0, nbp, A, lda, Vp);
        DCG_LAUNCHED(c);
        zgemm(c, OP_C, OP_N, nbp, nbp, m0, one, Vp, m0, 0, Vp, m0, 0, zero, G, nbp, 0, 1);
        wy_tfactor_kernel<<<1, WY_NB, 2 * WY_NB * WY_NB * sizeof(cplx), c.stream>>>(nbp, G, h.tau, k0, T);
        DCG_LAUNCHED(c);
        cplx *Zs = Z + (k0 + 1);
        zgemm(c, OP_C, OP_N, nbp, nvec, m0, one, Vp, m0, 0, Zs, ldz, 0, zero, W1, nbp, 0, 1);
        zgemm(c, OP_N, OP_N, nbp, nvec, nbp, one, T, WY_NB, 0, W1, nbp, 0, zero, W2, nbp, 0, 1);
        zgemm(c, OP_N, OP_N, m0, nvec, nbp, mone, Vp, m0, 0, W2, nbp, 0, one, Zs, ldz, 0, 1);
    }
}

void eig_slot_jobs(Context &c, const std::vector<VecJob> &vj, const std::vector<TE2Job> &tj) {
    struct Item {
        const VecJob *v;
        const TE2Job *t;
        double work;
    };
    std::vector<Item> items;
    double wv = 0.0, wt = 0.0;
    for (const VecJob &v : vj) {
        if (v.n <= 0 || v.vhi <= v.vlo || v.Z == nullptr) continue;
        if (v.n > 1024) {
            heev_vectors_slot(c, v.slot, v.n, v.A, v.lda, v.vlo, v.vhi, v.Z, v.ldz);
            continue;
        }
        const double w = 8.0 * (double)v.n * v.n * (v.vhi - v.vlo);
        items.push_back({&v, nullptr, w});
        wv += w;
    }
    for (const TE2Job &t : tj) {
        if (t.n <= 0 || t.nouter <= 0) continue;
        const double w = 8.0 * (double)t.n * t.n * t.nouter;
        items.push_back({nullptr, &t, w});
        wt += w;
    }
    if (items.empty()) return;
    std::stable_sort(items.begin(), items.end(), [](const Item &x, const Item &y) { return x.work > y.work; });
    FamScope fs(c, DCG_FAM_EIG, wv + wt);
    FamScope fb(c, DCG_FAM_EIG_BACK, wv);
    const int fam = c.fam;
    c.fam = 0;   // the two scopes above time the overlapped group once, on the context stream
    try {
        on_aux_streams(c, (int)items.size(), [&](int k) {
            const Item &it = items[k];
            if (it.v) heev_vectors_slot(c, it.v->slot, it.v->n, it.v->A, it.v->lda, it.v->vlo, it.v->vhi, it.v->Z, it.v->ldz);
            else tridiag_e2(c, it.t->slot, it.t->n, it.t->A, it.t->lda, it.t->VC, it.t->ldvc, it.t->nouter, it.t->alpha,
                            it.t->e2o, it.t->sco);
        });
    } catch (...) {
        c.fam = fam;
        throw;
    }
    c.fam = fam;
}

void heev(Context &c, int n, cplx *A, int64_t lda, double *w, int vlo, int vhi, cplx *Z, int64_t ldz) {
    if (n <= 0) return;
    EigJob j;
    j.n = n;
    j.A = A;
    j.lda = lda;
    j.w = w;
    j.slot = 0;
    heev_values_batched(c, std::vector<EigJob>(1, j));
    heev_vectors_slot(c, 0, n, A, lda, vlo, vhi, Z, ldz);
}

// Eigenvectors [vlo, vhi) of the matrix most recently passed to heev() (slot 0).
void heev_vectors_only(Context &c, int n, cplx *A, int64_t lda, const double *w, int vlo, int vhi, cplx *Z,
                       int64_t ldz) {
    (void)w;
    heev_vectors_slot(c, 0, n, A, lda, vlo, vhi, Z, ldz);
}

// Symmetric tridiagonal eigendecomposition (the divide-and-conquer stage alone): d (n),
// e (n-1) device arrays; ascending eigenvalues into w (device) and eigenvectors returned
// (device, n x n, ld n; valid until the next eigensolver call).
const double *stedc(Context &c, int n, const double *d, const double *e, double *w) {
    if (n <= 0) return nullptr;
    const double *Q = tridiag_dc(c, n, d, e, w, 0);
    check_dc_status(c, 0);
    return Q;
}

}  // namespace dcg

namespace dcg {
// Joint-launch counters of the merged reductions on a device: launches, launches that carried
// more than one context's submission, and submissions carried.
void coop_merge_stats(int device, int64_t out[3]) {
    out[0] = out[1] = out[2] = 0;
    std::lock_guard<std::mutex> lk(g_batchers_mu);
    auto it = g_batchers.find(device);
    if (it == g_batchers.end()) return;
    std::lock_guard<std::mutex> lb(it->second->mu);
    out[0] = it->second->launches;
    out[1] = it->second->joint;
    out[2] = it->second->carried;
}
}  // namespace dcg
