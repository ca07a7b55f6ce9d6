// Block Davidson eigensolver for the lowest roots of the CASCI Hamiltonian (Davidson,
// J. Comput. Phys. 17, 87 (1975); block form of Liu, 1978), the large-ndet CASCI route that
// replaces the dense ZHEEV of casci.F90:55-70 (diag.F90:66-128) when only a few roots are
// wanted.  The Hamiltonian stays in HBM as CSR (the diagonal and the single and double
// excitations of each determinant, dcg_ci.cu); every step is a device kernel:
//   W = H V                        (the sigma vectors, one warp per row of H)
//   G = V^H W                      (Rayleigh matrix, symmetrised)
//   G Y = Y diag(theta)            (one-block cyclic Jacobi, below)
//   R = W Y - V Y diag(theta)      (residuals of the block's Ritz pairs)
//   T = R / (theta - diag(H))      (diagonal preconditioner)
//   T orthonormalised against V    (classical Gram-Schmidt applied twice), appended to V.
// The host only orchestrates: per step it reads the residual norms and the lengths of the
// new directions back.  Converged when every wanted root has |r| <= tol.
#include <algorithm>
#include <cmath>
#include <functional>
#include <numeric>
#include <vector>

#include "dcg_common.cuh"
#include "dcg_kernels.cuh"

namespace dcg {

namespace {

constexpr int kJacobiMaxN = 64;
constexpr int kJacobiThreads = 256;
constexpr int kJacobiMaxSweeps = 40;

__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ double block_sum_d(double v, double *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    v = warp_sum_d(v);
    __syncthreads();
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    const int nw = (blockDim.x + 31) >> 5;
    double t = (threadIdx.x < nw) ? sh[threadIdx.x] : 0.0;
    if (wid == 0) t = warp_sum_d(t);
    if (threadIdx.x == 0) sh[0] = t;
    __syncthreads();
    const double r = sh[0];
    __syncthreads();
    return r;
}

// Player at position `pos` of round `s` of a round-robin tournament of np players (np even):
// position 0 stays, the others rotate.  Round s pairs positions k and np-1-k.
__device__ __forceinline__ int rr_player(int pos, int s, int np) {
    return pos == 0 ? 0 : 1 + (pos - 1 + s) % (np - 1);
}

// All eigenpairs of a small Hermitian matrix G (n <= 64, column-major, ldg; the matrix used is
// (G + G^H)/2) by cyclic Jacobi with the parallel round-robin ordering (Golub & Van Loan,
// Matrix Computations, 4th ed., 8.5.5): each round rotates n/2 disjoint pairs at once,
// A <- J^H A J, V <- V J.  The 2x2 Hermitian block [[a, |b| e^{i phi}], [., d]] is made real
// by the phase e^{i phi} and rotated by the symmetric Schur step (ibid. 8.5.2), so
// J_pp = J_qq = c, J_pq = s e^{i phi}, J_qp = -s e^{-i phi}.  Sweeps stop when the squared
// off-diagonal Frobenius norm is below 1e-30 of the whole (status 1 after 40 sweeps).
// Output: ascending eigenvalues w[n], eigenvectors Y (n x n, ldy).  One block.
__global__ void __launch_bounds__(kJacobiThreads) jacobi_heev_kernel(int n, const cplx *__restrict__ G, int ldg,
                                                                       double *w, cplx *Y, int ldy, int *status) {
    extern __shared__ double2 jsm[];
    const int np = n + (n & 1);   // padded to even: the dummy player pairs with nobody
    cplx *A = jsm;                // np x np
    cplx *V = A + np * np;        // np x np
    __shared__ double cs_c[kJacobiMaxN / 2], cs_s[kJacobiMaxN / 2], cs_pr[kJacobiMaxN / 2], cs_pi[kJacobiMaxN / 2];
    __shared__ int cs_p[kJacobiMaxN / 2], cs_q[kJacobiMaxN / 2];
    __shared__ double red[32];
    __shared__ int rank_sh[kJacobiMaxN];
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int e = tid; e < np * np; e += nt) {
        const int i = e % np, j = e / np;
        cplx a = mk(0.0, 0.0);
        if (i < n && j < n) {
            const cplx x = G[i + (int64_t)ldg * j], y = G[j + (int64_t)ldg * i];
            a = mk(0.5 * (x.x + y.x), 0.5 * (x.y - y.y));
            if (i == j) a.y = 0.0;
        }
        A[e] = a;
        V[e] = mk(i == j ? 1.0 : 0.0, 0.0);
    }
    __syncthreads();
    double fro = 0.0;
    for (int e = tid; e < np * np; e += nt) fro += A[e].x * A[e].x + A[e].y * A[e].y;
    fro = block_sum_d(fro, red);
    const int npair = np / 2;
    int sweep = 0;
    for (; sweep < kJacobiMaxSweeps; sweep++) {
        double off = 0.0;
        for (int e = tid; e < np * np; e += nt)
            if (e % np != e / np) off += A[e].x * A[e].x + A[e].y * A[e].y;
        off = block_sum_d(off, red);
        if (off <= 1e-30 * fro || fro == 0.0) break;
        for (int s = 0; s < np - 1; s++) {
            // rotation parameters of each pair from the current A
            for (int k = tid; k < npair; k += nt) {
                int p = rr_player(k, s, np), q = rr_player(np - 1 - k, s, np);
                if (p > q) {
                    const int t = p;
                    p = q;
                    q = t;
                }
                cs_p[k] = p;
                cs_q[k] = q;
                double c = 1.0, sn = 0.0, pr = 1.0, pi = 0.0;
                const cplx b = A[p + np * q];
                const double ab = sqrt(b.x * b.x + b.y * b.y);
                if (q < n && ab > 0.0) {
                    const double app = A[p + np * p].x, aqq = A[q + np * q].x;
                    const double zeta = (aqq - app) / (2.0 * ab);
                    const double t = (zeta >= 0.0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
                    c = 1.0 / sqrt(1.0 + t * t);
                    sn = t * c;
                    pr = b.x / ab;
                    pi = b.y / ab;
                }
                cs_c[k] = c;
                cs_s[k] = sn;
                cs_pr[k] = pr;
                cs_pi[k] = pi;
            }
            __syncthreads();
            // columns: A <- A J, V <- V J
            for (int e = tid; e < np * npair; e += nt) {
                const int i = e % np, k = e / np;
                const int p = cs_p[k], q = cs_q[k];
                const double c = cs_c[k], sn = cs_s[k];
                const cplx sp = mk(sn * cs_pr[k], sn * cs_pi[k]);    // s e^{i phi}
                const cplx sm = mk(sn * cs_pr[k], -sn * cs_pi[k]);   // s e^{-i phi}
                const cplx ap = A[i + np * p], aq = A[i + np * q];
                A[i + np * p] = csub(mk(c * ap.x, c * ap.y), cmul(sm, aq));
                A[i + np * q] = cadd(cmul(sp, ap), mk(c * aq.x, c * aq.y));
                const cplx vp = V[i + np * p], vq = V[i + np * q];
                V[i + np * p] = csub(mk(c * vp.x, c * vp.y), cmul(sm, vq));
                V[i + np * q] = cadd(cmul(sp, vp), mk(c * vq.x, c * vq.y));
            }
            __syncthreads();
            // rows: A <- J^H A
            for (int e = tid; e < np * npair; e += nt) {
                const int j = e % np, k = e / np;
                const int p = cs_p[k], q = cs_q[k];
                const double c = cs_c[k], sn = cs_s[k];
                const cplx sp = mk(sn * cs_pr[k], sn * cs_pi[k]);
                const cplx sm = mk(sn * cs_pr[k], -sn * cs_pi[k]);
                const cplx ap = A[p + np * j], aq = A[q + np * j];
                A[p + np * j] = csub(mk(c * ap.x, c * ap.y), cmul(sp, aq));
                A[q + np * j] = cadd(cmul(sm, ap), mk(c * aq.x, c * aq.y));
            }
            __syncthreads();
        }
    }
    // ascending order (ties by index), then the outputs
    for (int i = tid; i < n; i += nt) {
        const double di = A[i + np * i].x;
        int r = 0;
        for (int j = 0; j < n; j++) {
            const double dj = A[j + np * j].x;
            r += (dj < di) || (dj == di && j < i);
        }
        rank_sh[i] = r;
    }
    __syncthreads();
    for (int i = tid; i < n; i += nt) w[rank_sh[i]] = A[i + np * i].x;
    for (int e = tid; e < n * n; e += nt) {
        const int i = e % n, j = e / n;
        Y[i + (int64_t)ldy * rank_sh[j]] = V[i + np * j];
    }
    if (tid == 0) *status = sweep >= kJacobiMaxSweeps ? 1 : 0;
}

// Columns c of X (n x m) set to the unit vectors e_{idx[c]}.
__global__ void unit_cols_kernel(int n, int m, const int *__restrict__ idx, cplx *X, int64_t ldx) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)n * m) return;
    const int i = (int)(e % n), c = (int)(e / n);
    X[i + ldx * c] = mk(i == idx[c] ? 1.0 : 0.0, 0.0);
}

// R[:, c] = HX[:, c] - theta[c] X[:, c]; out2[c] = |R[:, c]|^2 (one block per column, fixed
// reduction order); T[:, c] = R[:, c] / (theta[c] - hd) with the denominator kept away from 0.
__global__ void residual_kernel(int n, const cplx *__restrict__ HX, const cplx *__restrict__ X, int64_t ld,
                                const double *__restrict__ theta, const double *__restrict__ hd, cplx *T,
                                double *out2) {
    __shared__ double sh[32];
    const int c = blockIdx.x;
    const double th = theta[c];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const cplx hx = HX[i + ld * c], x = X[i + ld * c];
        const cplx r = mk(hx.x - th * x.x, hx.y - th * x.y);
        acc += r.x * r.x + r.y * r.y;
        double den = th - hd[i];
        if (fabs(den) < 1e-4) den = den < 0.0 ? -1e-4 : 1e-4;
        T[i + ld * c] = mk(r.x / den, r.y / den);
    }
    acc = block_sum_d(acc, sh);
    if (threadIdx.x == 0) out2[c] = acc;
}

// out2[0] = |x|^2 (one block, fixed reduction order)
__global__ void norm2_kernel(int n, const cplx *__restrict__ x, double *out2) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += x[i].x * x[i].x + x[i].y * x[i].y;
    acc = block_sum_d(acc, sh);
    if (threadIdx.x == 0) out2[0] = acc;
}

// x <- x / sqrt(*n2)
__global__ void normalize_kernel(int n, cplx *x, const double *__restrict__ n2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double s = 1.0 / sqrt(*n2);
    x[i] = mk(x[i].x * s, x[i].y * s);
}

// C[i + ldc j] (op)= sum_k conj(A[k + lda i]) B[k + ldb j] for a small i x j output and a long
// k: one block per output element, fixed-order reduction.  beta: 0 overwrite, 1 accumulate
// with alpha.
__global__ void dotc_small_kernel(int n, const cplx *__restrict__ A, int64_t lda, const cplx *__restrict__ B,
                                  int64_t ldb, cplx *C, int ldc, double alpha, int accumulate) {
    __shared__ double sh[32];
    const int i = blockIdx.x, j = blockIdx.y;
    const cplx *a = A + lda * i, *b = B + ldb * j;
    double re = 0.0, im = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const cplx x = a[k], y = b[k];
        re += x.x * y.x + x.y * y.y;
        im += x.x * y.y - x.y * y.x;
    }
    re = block_sum_d(re, sh);
    im = block_sum_d(im, sh);
    if (threadIdx.x == 0) {
        cplx v = mk(alpha * re, alpha * im);
        if (accumulate) v = cadd(v, C[i + (int64_t)ldc * j]);
        C[i + (int64_t)ldc * j] = v;
    }
}

// C (n x k) = alpha A (n x m) B (m x k) + beta C, m and k small: one thread per row (coalesced
// over rows), the m x k factor read through the read-only cache.
__global__ void tall_small_kernel(int n, int m, int k, cplx alpha, const cplx *__restrict__ A, int64_t lda,
                                  const cplx *__restrict__ B, int ldb, cplx beta, cplx *C, int64_t ldc) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int c = blockIdx.y;
    if (r >= n) return;
    cplx acc = mk(0.0, 0.0);
    for (int q = 0; q < m; q++) acc = cadd(acc, cmul(A[r + lda * q], __ldg(B + q + (int64_t)ldb * c)));
    cplx v = cmul(alpha, acc);
    if (beta.x != 0.0 || beta.y != 0.0) v = cadd(v, cmul(beta, C[r + ldc * c]));
    C[r + ldc * c] = v;
}

// Y[:, c] = H X[:, c] for K vectors and a CSR H: one warp per row, the lanes striding the row's
// entries in order and a fixed shuffle tree summing them (deterministic).
template <int K>
__global__ void __launch_bounds__(256) csr_hx_kernel(int n, int k, const int64_t *__restrict__ rowptr,
                                                      const int *__restrict__ cols, const cplx *__restrict__ vals,
                                                      const cplx *__restrict__ X, int64_t ldx, cplx *Y, int64_t ldy) {
    const int row = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    if (row >= n) return;
    double re[K], im[K];
#pragma unroll
    for (int c = 0; c < K; c++) re[c] = im[c] = 0.0;
    const int64_t e1 = rowptr[row + 1];
    for (int64_t e = rowptr[row] + lane; e < e1; e += 32) {
        const cplx h = vals[e];
        const int j = cols[e];
#pragma unroll
        for (int c = 0; c < K; c++) {
            if (c < k) {
                const cplx x = __ldg(X + j + ldx * c);
                re[c] = fma(h.x, x.x, fma(-h.y, x.y, re[c]));
                im[c] = fma(h.x, x.y, fma(h.y, x.x, im[c]));
            }
        }
    }
#pragma unroll
    for (int c = 0; c < K; c++) {
        for (int o = 16; o > 0; o >>= 1) {
            re[c] += __shfl_down_sync(0xffffffffu, re[c], o);
            im[c] += __shfl_down_sync(0xffffffffu, im[c], o);
        }
    }
    if (lane == 0) {
#pragma unroll
        for (int c = 0; c < K; c++)
            if (c < k) Y[row + ldy * c] = mk(re[c], im[c]);
    }
}

}  // namespace

// C (mi x mj, ldc) = A^H B over n rows (Davidson inner products).
static void dotc_small(Context &c, int n, int mi, int mj, const cplx *A, int64_t lda, const cplx *B, int64_t ldb,
                       cplx *C, int ldc, double alpha = 1.0, bool accumulate = false) {
    if (mi <= 0 || mj <= 0) return;
    dotc_small_kernel<<<dim3(mi, mj), 256, 0, c.stream>>>(n, A, lda, B, ldb, C, ldc, alpha, accumulate ? 1 : 0);
    DCG_LAUNCHED(c);
}

static void tall_small(Context &c, int n, int m, int k, cplx alpha, const cplx *A, int64_t lda, const cplx *B, int ldb,
                       cplx beta, cplx *C, int64_t ldc) {
    if (n <= 0 || k <= 0) return;
    tall_small_kernel<<<dim3(grid1d(n, 128), k), 128, 0, c.stream>>>(n, m, k, alpha, A, lda, B, ldb, beta, C, ldc);
    DCG_LAUNCHED(c);
}

// Y (n x k) = H X for the CSR H, up to 8 vectors a launch (one pass over H for each group).
static void csr_hx(Context &c, const CsrMatrix &H, const cplx *X, int64_t ldx, int k, cplx *Y, int64_t ldy) {
    const int n = H.n;
    const int blocks = (int)(((int64_t)n * 32 + 255) / 256);
    for (int c0 = 0; c0 < k; c0 += 8) {
        const int kk = std::min(8, k - c0);
        if (kk > 4)
            csr_hx_kernel<8><<<blocks, 256, 0, c.stream>>>(n, kk, H.rowptr, H.cols, H.vals, X + ldx * c0, ldx,
                                                            Y + ldy * c0, ldy);
        else if (kk > 2)
            csr_hx_kernel<4><<<blocks, 256, 0, c.stream>>>(n, kk, H.rowptr, H.cols, H.vals, X + ldx * c0, ldx,
                                                            Y + ldy * c0, ldy);
        else
            csr_hx_kernel<2><<<blocks, 256, 0, c.stream>>>(n, kk, H.rowptr, H.cols, H.vals, X + ldx * c0, ldx,
                                                            Y + ldy * c0, ldy);
        DCG_LAUNCHED(c);
    }
}

void small_heev(Context &c, int n, const cplx *G, int ldg, double *w, cplx *Y, int ldy) {
    if (n < 1 || n > kJacobiMaxN) throw Error{DCG_E_ARG, "small_heev: dimension out of range"};
    const int np = n + (n & 1);
    const size_t smem = 2 * sizeof(cplx) * (size_t)np * np;
    DCG_CUDA(cudaFuncSetAttribute(jacobi_heev_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int *st = wsget<int>(c, "dav.jst", 1);
    // two warps: the rounds are short (n/2 rotations), so barrier latency, not work, sets the pace
    jacobi_heev_kernel<<<1, 64, smem, c.stream>>>(n, G, ldg, w, Y, ldy, st);
    DCG_LAUNCHED(c);
}

using HxFn = std::function<void(const cplx *X, int64_t ldx, int k, cplx *Y, int64_t ldy)>;

// Block Davidson on the operator hx (Y = H X) with diagonal hd (device, n).
static void davidson_core(Context &c, int n, const HxFn &hx, const double *hd, int nwant, double *w, cplx *Z,
                          double tol_rel, int maxit) {
    const int nb = std::min(n, nwant + 2);   // block: the wanted roots and a margin for near-degeneracy
    const int mmax = std::min(n, std::min(kJacobiMaxN, std::max(24, 8 * nb)));
    if (nwant < 1 || nb > mmax || n < 2) throw Error{DCG_E_ARG, "davidson: block does not fit the subspace"};
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0), mone = mk(-1.0, 0.0);
    const int64_t ld = n;
    cplx *V = wsget<cplx>(c, "dav.V", (size_t)n * mmax);
    cplx *W = wsget<cplx>(c, "dav.W", (size_t)n * mmax);
    cplx *X = wsget<cplx>(c, "dav.X", (size_t)n * nb);
    cplx *HX = wsget<cplx>(c, "dav.HX", (size_t)n * nb);
    cplx *T = wsget<cplx>(c, "dav.T", (size_t)n * nb);
    cplx *G = wsget<cplx>(c, "dav.G", (size_t)mmax * mmax);
    cplx *Y = wsget<cplx>(c, "dav.Y", (size_t)mmax * mmax);
    cplx *cf = wsget<cplx>(c, "dav.cf", (size_t)mmax);
    double *th = wsget<double>(c, "dav.th", mmax);
    double *nrm = wsget<double>(c, "dav.nrm", (size_t)3 * nb);
    int *idx = wsget<int>(c, "dav.idx", nb);
    int *jst = wsget<int>(c, "dav.jst", 1);

    // start: unit vectors on the nb lowest diagonal elements (ties by index)
    std::vector<double> hdh(n);
    DCG_CUDA(cudaMemcpyAsync(hdh.data(), hd, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
    DCG_CUDA(cudaStreamSynchronize(c.stream));
    double hscale = 1.0;
    for (double x : hdh) hscale = std::max(hscale, std::fabs(x));
    const double tol = tol_rel * hscale;
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::partial_sort(order.begin(), order.begin() + nb, order.end(),
                      [&](int a, int b) { return hdh[a] < hdh[b] || (hdh[a] == hdh[b] && a < b); });
    DCG_CUDA(cudaMemcpyAsync(idx, order.data(), sizeof(int) * nb, cudaMemcpyHostToDevice, c.stream));
    unit_cols_kernel<<<grid1d((int64_t)n * nb, 256), 256, 0, c.stream>>>(n, nb, idx, V, ld);
    DCG_LAUNCHED(c);
    int m = nb;
    hx(V, ld, m, W, ld);

    std::vector<double> h2((size_t)nb);
    bool converged = false;
    c.casci_iters = 0;
    for (int it = 0; it < maxit; it++) {
        dotc_small(c, n, m, m, V, ld, W, ld, G, mmax);
        small_heev(c, m, G, mmax, th, Y, mmax);
        // Ritz vectors of the block and their images
        tall_small(c, n, m, nb, one, V, ld, Y, mmax, zero, X, ld);
        tall_small(c, n, m, nb, one, W, ld, Y, mmax, zero, HX, ld);
        residual_kernel<<<nb, 256, 0, c.stream>>>(n, HX, X, ld, th, hd, T, nrm);
        DCG_LAUNCHED(c);
        DCG_CUDA(cudaMemcpyAsync(h2.data(), nrm, sizeof(double) * nb, cudaMemcpyDeviceToHost, c.stream));
        DCG_CUDA(cudaStreamSynchronize(c.stream));
        c.casci_iters = it + 1;
        double worst = 0.0;
        for (int q = 0; q < nwant; q++) worst = std::max(worst, std::sqrt(h2[q]));
        if (worst <= tol) {
            converged = true;
            break;
        }
        if (m + nb > mmax) {   // restart on the block's Ritz vectors (orthonormal)
            DCG_CUDA(cudaMemcpyAsync(V, X, sizeof(cplx) * (size_t)n * nb, cudaMemcpyDeviceToDevice, c.stream));
            DCG_CUDA(cudaMemcpyAsync(W, HX, sizeof(cplx) * (size_t)n * nb, cudaMemcpyDeviceToDevice, c.stream));
            m = nb;
        }
        // new directions: preconditioned residuals of the unconverged Ritz pairs, made
        // orthonormal to V and to each other (classical Gram-Schmidt, twice) on the device; the
        // norms before and after come back in one read, and a direction that has lost all but
        // 1e-10 of its length ends the block there
        int cand = 0;
        for (int q = 0; q < nb && m + cand < mmax; q++) {
            if (std::sqrt(h2[q]) <= tol) continue;
            cplx *dst = V + ld * (m + cand);
            DCG_CUDA(cudaMemcpyAsync(dst, T + ld * q, sizeof(cplx) * n, cudaMemcpyDeviceToDevice, c.stream));
            norm2_kernel<<<1, 256, 0, c.stream>>>(n, dst, nrm + nb + 2 * cand);
            DCG_LAUNCHED(c);
            const int mm = m + cand;
            for (int pass = 0; pass < 2; pass++) {
                dotc_small(c, n, mm, 1, V, ld, dst, ld, cf, mmax);
                tall_small(c, n, mm, 1, mone, V, ld, cf, mmax, one, dst, ld);
            }
            norm2_kernel<<<1, 256, 0, c.stream>>>(n, dst, nrm + nb + 2 * cand + 1);
            DCG_LAUNCHED(c);
            normalize_kernel<<<grid1d(n, 256), 256, 0, c.stream>>>(n, dst, nrm + nb + 2 * cand + 1);
            DCG_LAUNCHED(c);
            cand++;
        }
        int added = 0;
        if (cand > 0) {
            std::vector<double> nn((size_t)2 * cand);
            DCG_CUDA(cudaMemcpyAsync(nn.data(), nrm + nb, sizeof(double) * 2 * cand, cudaMemcpyDeviceToHost,
                                     c.stream));
            DCG_CUDA(cudaStreamSynchronize(c.stream));
            while (added < cand && nn[2 * added + 1] > 1e-20 * nn[2 * added] && nn[2 * added + 1] > 0.0) added++;
        }
        if (added == 0) break;   // stagnated: reported below
        hx(V + ld * m, ld, added, W + ld * m, ld);
        m += added;
    }
    int jh = 0;
    DCG_CUDA(cudaMemcpyAsync(&jh, jst, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    DCG_CUDA(cudaStreamSynchronize(c.stream));
    if (!converged || jh != 0)
        throw Error{DCG_E_NUMERIC, "CASCI Davidson did not converge to |r| <= " + std::to_string(tol)};
    DCG_CUDA(cudaMemcpyAsync(w, th, sizeof(double) * nwant, cudaMemcpyDeviceToDevice, c.stream));
    DCG_CUDA(cudaMemcpyAsync(Z, X, sizeof(cplx) * (size_t)n * nwant, cudaMemcpyDeviceToDevice, c.stream));
}

// Lowest nwant eigenpairs of the Hermitian CSR H (its diagonal kept beside it): eigenvalues to
// w[0..nwant), eigenvectors to the columns of Z (n x nwant, ldz = n), each with residual norm
// <= tol_rel * max(1, max_i |H_ii|).
void davidson_lowest_csr(Context &c, const CsrMatrix &H, int nwant, double *w, cplx *Z, double tol_rel, int maxit) {
    davidson_core(
        c, H.n, [&](const cplx *X, int64_t ldx, int k, cplx *Y, int64_t ldy) { csr_hx(c, H, X, ldx, k, Y, ldy); },
        H.diag, nwant, w, Z, tol_rel, maxit);
}

}  // namespace dcg
