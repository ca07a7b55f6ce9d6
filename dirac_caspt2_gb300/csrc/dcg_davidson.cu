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
__global__ void __launch_bounds__(kJacobiThreads) jacobi_heev_kernel(int n, const int *__restrict__ n_dev,
                                                                       const cplx *__restrict__ G, int ldg,
                                                                       double *w, cplx *Y, int ldy, int *status) {
    extern __shared__ double2 jsm[];
    if (n_dev) n = *n_dev;   // dimension read on the device (graph replays of a Davidson step)
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
                const double ab2 = b.x * b.x + b.y * b.y;
                // a rotation whose off-diagonal element is below 1e-34 of the squared norm is
                // skipped (all of them together stay under the 1e-30 stopping test): the late
                // sweeps of the quadratic convergence then cost little FP64 work
                if (q < n && ab2 > 1e-34 * fro) {
                    const double ab = sqrt(ab2);
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
            // columns: A <- A J, V <- V J (identity rotations skipped)
            for (int e = tid; e < np * npair; e += nt) {
                const int i = e % np, k = e / np;
                const double c = cs_c[k], sn = cs_s[k];
                if (sn == 0.0) continue;
                const int p = cs_p[k], q = cs_q[k];
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
                const double c = cs_c[k], sn = cs_s[k];
                if (sn == 0.0) continue;
                const int p = cs_p[k], q = cs_q[k];
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
    if (tid == 0 && sweep >= kJacobiMaxSweeps) *status = 1;
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

// ---- the Davidson step with its sizes on the device ------------------------------------
// A step's launches read the subspace size m and the running counts from DavState, so one
// captured sequence (a CUDA graph) serves every step.
struct DavState {
    int m;        // vectors in V (and W = H V)
    int cand;     // new directions accepted in this step
    int stop;     // a direction was rejected: none after it this step
    int act;      // the direction being built is live
    int jac;      // a Jacobi solve ran out of sweeps (sticky)
    int pad[3];
    double worst;  // largest residual norm of the wanted roots
    double n0;     // |direction|^2 before the Gram-Schmidt passes
};

// G[i + ldg j] = V[:, i]^H W[:, j] for i, j < m (one block per element, fixed order).
__global__ void rr_kernel(int n, const cplx *__restrict__ V, const cplx *__restrict__ W, int64_t ld, cplx *G,
                          int ldg, const DavState *__restrict__ st) {
    __shared__ double sh[32];
    const int i = blockIdx.x, j = blockIdx.y, m = st->m;
    if (i >= m || j >= m) return;
    const cplx *a = V + ld * i, *b = W + ld * j;
    double re = 0.0, im = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const cplx x = a[k], y = b[k];
        re += x.x * y.x + x.y * y.y;
        im += x.x * y.y - x.y * y.x;
    }
    re = block_sum_d(re, sh);
    im = block_sum_d(im, sh);
    if (threadIdx.x == 0) G[i + (int64_t)ldg * j] = mk(re, im);
}

// X = V Y[:, :nb] (z = 0) and HX = W Y[:, :nb] (z = 1) over the m columns of V and W.
__global__ void ritz_kernel(int n, const cplx *__restrict__ V, const cplx *__restrict__ W, int64_t ld,
                            const cplx *__restrict__ Y, int ldy, cplx *X, cplx *HX, const DavState *__restrict__ st) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    if (r >= n) return;
    const cplx *A = blockIdx.z ? W : V;
    const int m = st->m;
    cplx acc = mk(0.0, 0.0);
    for (int q = 0; q < m; q++) acc = cadd(acc, cmul(A[r + ld * q], __ldg(Y + q + (int64_t)ldy * c)));
    (blockIdx.z ? HX : X)[r + ld * c] = acc;
}

// The residual norms of the wanted roots; the step's direction counters reset.
__global__ void step_begin_kernel(int nwant, const double *__restrict__ h2, DavState *st) {
    if (threadIdx.x != 0) return;
    double w = 0.0;
    for (int q = 0; q < nwant; q++) w = fmax(w, sqrt(h2[q]));
    st->worst = w;
    st->cand = 0;
    st->stop = 0;
}

// Restart on the block's Ritz vectors when the next block would not fit: V, W <- X, HX.
__global__ void restart_copy_kernel(int n, int nb, int mmax, const cplx *__restrict__ X, const cplx *__restrict__ HX,
                                    cplx *V, cplx *W, int64_t ld, const DavState *__restrict__ st) {
    if (st->m + nb <= mmax) return;
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)n * nb) return;
    const int i = (int)(e % n), c = (int)(e / n);
    V[i + ld * c] = X[i + ld * c];
    W[i + ld * c] = HX[i + ld * c];
}

__global__ void restart_set_kernel(int nb, int mmax, DavState *st) {
    if (threadIdx.x == 0 && st->m + nb > mmax) st->m = nb;
}

// Direction q: live when its residual is above tol, the block has not stopped and V has room;
// then T[:, q] goes to column m + cand of V and its squared norm to n0 (one block).
__global__ void cand_begin_kernel(int n, int q, int mmax, double tol, const double *__restrict__ h2,
                                  const cplx *__restrict__ T, cplx *V, int64_t ld, DavState *st) {
    __shared__ double sh[32];
    __shared__ int live;
    if (threadIdx.x == 0) {
        live = !st->stop && sqrt(h2[q]) > tol && st->m + st->cand < mmax;
        st->act = live;
    }
    __syncthreads();
    if (!live) return;
    cplx *dst = V + ld * (st->m + st->cand);
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const cplx x = T[i + ld * q];
        dst[i] = x;
        acc += x.x * x.x + x.y * x.y;
    }
    acc = block_sum_d(acc, sh);
    if (threadIdx.x == 0) st->n0 = acc;
}

// Classical Gram-Schmidt pass of the live direction against the vectors before it.
__global__ void cgs_dot_kernel(int n, const cplx *__restrict__ V, int64_t ld, cplx *cf, const DavState *__restrict__ st) {
    __shared__ double sh[32];
    const int i = blockIdx.x, mm = st->m + st->cand;
    if (!st->act || i >= mm) return;
    const cplx *a = V + ld * i, *b = V + ld * mm;
    double re = 0.0, im = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const cplx x = a[k], y = b[k];
        re += x.x * y.x + x.y * y.y;
        im += x.x * y.y - x.y * y.x;
    }
    re = block_sum_d(re, sh);
    im = block_sum_d(im, sh);
    if (threadIdx.x == 0) cf[i] = mk(re, im);
}

__global__ void cgs_axpy_kernel(int n, cplx *V, int64_t ld, const cplx *__restrict__ cf, const DavState *__restrict__ st) {
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    const int mm = st->m + st->cand;
    if (!st->act || r >= n) return;
    cplx acc = mk(0.0, 0.0);
    for (int q = 0; q < mm; q++) acc = cadd(acc, cmul(V[r + ld * q], cf[q]));
    cplx &d = V[r + ld * mm];
    d = csub(d, acc);
}

// Accept the live direction when it kept more than 1e-10 of its length (normalised, counted),
// else stop the block's directions here.
__global__ void cand_end_kernel(int n, cplx *V, int64_t ld, DavState *st) {
    __shared__ double sh[32];
    if (!st->act) return;
    cplx *dst = V + ld * (st->m + st->cand);
    double acc = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc += dst[i].x * dst[i].x + dst[i].y * dst[i].y;
    acc = block_sum_d(acc, sh);
    const bool ok = acc > 1e-20 * st->n0 && acc > 0.0;
    if (ok) {
        const double s = 1.0 / sqrt(acc);
        for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = mk(dst[i].x * s, dst[i].y * s);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        if (ok) st->cand++;
        else st->stop = 1;
    }
}

// W[:, m + c] = H V[:, m + c] for the cand accepted directions (CSR, one warp per row).
template <int K>
__global__ void __launch_bounds__(256) csr_hx_step_kernel(int n, const int64_t *__restrict__ rowptr,
                                                           const int *__restrict__ cols, const cplx *__restrict__ vals,
                                                           const cplx *__restrict__ V, cplx *W, int64_t ld,
                                                           const DavState *__restrict__ st) {
    const int row = (int)(((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int lane = threadIdx.x & 31;
    const int k = st->cand;
    if (row >= n || k == 0) return;
    const cplx *X = V + ld * st->m;
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
                const cplx x = __ldg(X + j + ld * c);
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
        cplx *Y = W + ld * st->m;
#pragma unroll
        for (int c = 0; c < K; c++)
            if (c < k) Y[row + ld * c] = mk(re[c], im[c]);
    }
}

__global__ void step_end_kernel(DavState *st) {
    if (threadIdx.x == 0) st->m += st->cand;
}

}  // namespace

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

// Lowest nwant eigenpairs of the Hermitian CSR H (its diagonal kept beside it): eigenvalues to
// w[0..nwant), eigenvectors to the columns of Z (n x nwant, ldz = n), each with residual norm
// <= tol_rel * max(1, max_i |H_ii|).
//
// One step: the Rayleigh matrix G = V^H W and its eigenpairs (Jacobi), the block's Ritz
// vectors X = V Y and images HX = W Y, their residuals and preconditioned corrections T, a
// restart V, W <- X, HX when the next block would not fit, then each unconverged correction
// orthonormalised against V (classical Gram-Schmidt twice) and appended, and W extended by
// H times the new directions.  Every size the step needs lives on the device (DavState), so
// the step is one fixed launch sequence: captured once as a CUDA graph and replayed, with
// one read of the state per step (the environment variable DCG_DAVIDSON_GRAPH=0 launches
// the sequence directly instead).
void davidson_lowest_csr(Context &c, const CsrMatrix &H, int nwant, double *w, cplx *Z, double tol_rel, int maxit) {
    const int n = H.n;
    const int nb = std::min(n, nwant + 2);   // block: the wanted roots and a margin for near-degeneracy
    const int mmax = std::min(n, std::min(kJacobiMaxN, std::max(24, 8 * nb)));
    if (nwant < 1 || nb > mmax || n < 2) throw Error{DCG_E_ARG, "davidson: block does not fit the subspace"};
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
    double *h2 = wsget<double>(c, "dav.h2", (size_t)nb);
    int *idx = wsget<int>(c, "dav.idx", nb);
    DavState *st = wsget<DavState>(c, "dav.st", 1);
    DavState *hst = reinterpret_cast<DavState *>(c.ws.host("dav.hst", sizeof(DavState)));

    // start: unit vectors on the nb lowest diagonal elements (ties by index)
    std::vector<double> hdh(n);
    DCG_CUDA(cudaMemcpyAsync(hdh.data(), H.diag, sizeof(double) * n, cudaMemcpyDeviceToHost, c.stream));
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
    csr_hx(c, H, V, ld, nb, W, ld);
    DavState s0{};
    s0.m = nb;
    DCG_CUDA(cudaMemcpyAsync(st, &s0, sizeof(DavState), cudaMemcpyHostToDevice, c.stream));

    const int np = mmax + (mmax & 1);
    const size_t jsmem = 2 * sizeof(cplx) * (size_t)np * np;
    DCG_CUDA(cudaFuncSetAttribute(jacobi_heev_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)jsmem));
    const int hx_blocks = (int)(((int64_t)n * 32 + 255) / 256);
    auto enqueue_step = [&]() {
        rr_kernel<<<dim3(mmax, mmax), 256, 0, c.stream>>>(n, V, W, ld, G, mmax, st);
        jacobi_heev_kernel<<<1, kJacobiThreads, jsmem, c.stream>>>(mmax, &st->m, G, mmax, th, Y, mmax, &st->jac);
        ritz_kernel<<<dim3(grid1d(n, 128), nb, 2), 128, 0, c.stream>>>(n, V, W, ld, Y, mmax, X, HX, st);
        residual_kernel<<<nb, 256, 0, c.stream>>>(n, HX, X, ld, th, H.diag, T, h2);
        step_begin_kernel<<<1, 32, 0, c.stream>>>(nwant, h2, st);
        restart_copy_kernel<<<grid1d((int64_t)n * nb, 256), 256, 0, c.stream>>>(n, nb, mmax, X, HX, V, W, ld, st);
        restart_set_kernel<<<1, 32, 0, c.stream>>>(nb, mmax, st);
        for (int q = 0; q < nb; q++) {
            cand_begin_kernel<<<1, 256, 0, c.stream>>>(n, q, mmax, tol, h2, T, V, ld, st);
            for (int pass = 0; pass < 2; pass++) {
                cgs_dot_kernel<<<mmax, 256, 0, c.stream>>>(n, V, ld, cf, st);
                cgs_axpy_kernel<<<grid1d(n, 128), 128, 0, c.stream>>>(n, V, ld, cf, st);
            }
            cand_end_kernel<<<1, 256, 0, c.stream>>>(n, V, ld, st);
        }
        if (nb > 4)
            csr_hx_step_kernel<8><<<hx_blocks, 256, 0, c.stream>>>(n, H.rowptr, H.cols, H.vals, V, W, ld, st);
        else if (nb > 2)
            csr_hx_step_kernel<4><<<hx_blocks, 256, 0, c.stream>>>(n, H.rowptr, H.cols, H.vals, V, W, ld, st);
        else
            csr_hx_step_kernel<2><<<hx_blocks, 256, 0, c.stream>>>(n, H.rowptr, H.cols, H.vals, V, W, ld, st);
        step_end_kernel<<<1, 32, 0, c.stream>>>(st);
        DCG_CUDA(cudaMemcpyAsync(hst, st, sizeof(DavState), cudaMemcpyDeviceToHost, c.stream));
    };
    const int step_kernels = 9 + 6 * nb;   // kernels per step
    if (nb > 8) throw Error{DCG_E_ARG, "davidson: more than 8 directions per step"};

    static const bool use_graph = [] {
        const char *e = getenv("DCG_DAVIDSON_GRAPH");
        return !(e && e[0] == '0');
    }();
    cudaGraphExec_t exec = nullptr;
    if (use_graph) {
        cudaGraph_t graph = nullptr;
        DCG_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step();
        DCG_CUDA(cudaStreamEndCapture(c.stream, &graph));
        const cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
        cudaGraphDestroy(graph);
        if (e != cudaSuccess) throw Error{DCG_E_CUDA, std::string("davidson graph: ") + cudaGetErrorString(e)};
    }
    struct ExecGuard {
        cudaGraphExec_t g;
        ~ExecGuard() {
            if (g) cudaGraphExecDestroy(g);
        }
    } guard{exec};

    bool converged = false;
    c.casci_iters = 0;
    for (int it = 0; it < maxit; it++) {
        if (exec) {
            DCG_CUDA(cudaGraphLaunch(exec, c.stream));
            c.launches += step_kernels;
        } else {
            enqueue_step();
            c.launches += step_kernels;
        }
        DCG_CUDA(cudaStreamSynchronize(c.stream));
        c.casci_iters = it + 1;
        if (hst->worst <= tol) {
            converged = true;
            break;
        }
        if (hst->cand == 0) break;   // stagnated: reported below
    }
    if (!converged || hst->jac != 0)
        throw Error{DCG_E_NUMERIC, "CASCI Davidson did not converge to |r| <= " + std::to_string(tol)};
    DCG_CUDA(cudaMemcpyAsync(w, th, sizeof(double) * nwant, cudaMemcpyDeviceToDevice, c.stream));
    DCG_CUDA(cudaMemcpyAsync(Z, X, sizeof(cplx) * (size_t)n * nwant, cudaMemcpyDeviceToDevice, c.stream));
}

}  // namespace dcg
