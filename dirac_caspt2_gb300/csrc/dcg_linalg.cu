// Dense FP64 complex linear algebra on the device: GEMM, Hermitian eigensolver and LU
// solve.  Written from the textbook algorithms:
//   - Householder reduction of a Hermitian matrix to real symmetric tridiagonal form
//     (Golub & Van Loan, Matrix Computations, 4th ed., 8.3.1), with the complex
//     reflector of LAPACK's documented xLARFG definition (beta real);
//   - eigenvalues by Sturm-count bisection (GVL 8.4.1);
//   - eigenvectors by inverse iteration on the tridiagonal with partial-pivoting LU
//     (GVL 8.2.2), followed by modified Gram-Schmidt inside clusters of close eigenvalues;
//   - back-transformation by the stored reflectors.
// Eigenvalues come out ascending, as the reference's ZHEEV/DSYEV calls
// (src/diag.F90:43,109) return them.
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

void Workspace::release_all() {
    for (auto &kv : bufs_)
        if (kv.second.p) cudaFree(kv.second.p);
    bufs_.clear();
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
template <int OPA, int OPB>
__global__ void __launch_bounds__(256) zgemm_kernel(int m, int n, int k, cplx alpha, const cplx *__restrict__ A,
                                                    int64_t lda, int64_t sa, const cplx *__restrict__ B,
                                                    int64_t ldb, int64_t sb, cplx beta, cplx *C, int64_t ldc,
                                                    int64_t sc, int zoff) {
    constexpr int BM = 64, BN = 64, BK = 16;
    __shared__ cplx As[BK][BM + 1];
    __shared__ cplx Bs[BK][BN + 1];
    const int64_t bz = (int64_t)blockIdx.z + zoff;
    A += bz * sa;
    B += bz * sb;
    C += bz * sc;
    const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
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
                a[q] = As[kk][ty + 16 * q];
                b[q] = Bs[kk][tx + 16 * q];
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
        int gi = m0 + ty + 16 * p;
        if (gi >= m) continue;
#pragma unroll
        for (int q = 0; q < 4; q++) {
            int gj = n0 + tx + 16 * q;
            if (gj >= n) continue;
            cplx r = cmul(alpha, acc[p][q]);
            int64_t o = gi + (int64_t)gj * ldc;
            if (use_beta) r = cadd(r, cmul(beta, C[o]));
            C[o] = r;
        }
    }
}

template <int OPA, int OPB>
static void zgemm_launch(Context &c, int m, int n, int k, cplx alpha, const cplx *A, int64_t lda, int64_t sa,
                         const cplx *B, int64_t ldb, int64_t sb, cplx beta, cplx *C, int64_t ldc, int64_t sc,
                         int batch) {
    for (int z0 = 0; z0 < batch; z0 += 65535) {
        int nz = batch - z0 < 65535 ? batch - z0 : 65535;
        dim3 grid(grid1d(m, 64), grid1d(n, 64), nz);
        zgemm_kernel<OPA, OPB><<<grid, 256, 0, c.stream>>>(m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc,
                                                           sc, z0);
        DCG_LAUNCHED(c);
    }
}

void zgemm(Context &c, Op opa, Op opb, int m, int n, int k, cplx alpha, const cplx *A, int64_t lda, int64_t sa,
           const cplx *B, int64_t ldb, int64_t sb, cplx beta, cplx *C, int64_t ldc, int64_t sc, int batch) {
    if (m <= 0 || n <= 0 || batch <= 0) return;
    if (k <= 0) {
        // C = beta*C : run with k=0 through the kernel (acc stays zero)
    }
#define DCG_ZG(a, b)                                                                                   \
    if (opa == a && opb == b) {                                                                        \
        zgemm_launch<a, b>(c, m, n, k, alpha, A, lda, sa, B, ldb, sb, beta, C, ldc, sc, batch);        \
        return;                                                                                        \
    }
    DCG_ZG(OP_N, OP_N) DCG_ZG(OP_N, OP_T) DCG_ZG(OP_N, OP_C) DCG_ZG(OP_N, OP_R)
    DCG_ZG(OP_T, OP_N) DCG_ZG(OP_T, OP_T) DCG_ZG(OP_T, OP_C) DCG_ZG(OP_T, OP_R)
    DCG_ZG(OP_C, OP_N) DCG_ZG(OP_C, OP_T) DCG_ZG(OP_C, OP_C) DCG_ZG(OP_C, OP_R)
    DCG_ZG(OP_R, OP_N) DCG_ZG(OP_R, OP_T) DCG_ZG(OP_R, OP_C) DCG_ZG(OP_R, OP_R)
#undef DCG_ZG
    throw Error{DCG_E_ARG, "zgemm: bad op"};
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

void dsum(Context &c, const double *x, int64_t n, double *out) {
    dsum_kernel<<<1, 1024, 0, c.stream>>>(x, n, out);
    DCG_LAUNCHED(c);
}

// ===================================================================== tridiagonalisation
// Step k: reflector for column k (rows k+1..n-1), v stored in A(k+1:n-1, k) with v0 = 1.
__global__ void hh_gen_kernel(int n, int k, cplx *A, int64_t lda, double *d, double *e, cplx *tau) {
    __shared__ double sh[32];
    __shared__ cplx s_scale;
    __shared__ int s_skip;
    const int m = n - k - 1;
    cplx *x = A + (k + 1) + (int64_t)k * lda;
    double s = 0.0;
    for (int i = 1 + threadIdx.x; i < m; i += blockDim.x) s += cabs2(x[i]);
    s = block_sum(s, sh);
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
    sr = block_sum(sr, sh);
    si = block_sum(si, sh);
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

// Gershgorin interval of the tridiagonal -> bounds[0..1]; also max |T| in bounds[2]
__global__ void gersh_kernel(int n, const double *d, const double *e, double *bounds) {
    __shared__ double lo_s[1024], hi_s[1024];
    double lo = 1e300, hi = -1e300;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double r = 0.0;
        if (i > 0) r += fabs(e[i - 1]);
        if (i < n - 1) r += fabs(e[i]);
        lo = fmin(lo, d[i] - r);
        hi = fmax(hi, d[i] + r);
    }
    lo_s[threadIdx.x] = lo;
    hi_s[threadIdx.x] = hi;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) {
            lo_s[threadIdx.x] = fmin(lo_s[threadIdx.x], lo_s[threadIdx.x + s]);
            hi_s[threadIdx.x] = fmax(hi_s[threadIdx.x], hi_s[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double L = lo_s[0], H = hi_s[0];
        double tn = fmax(fabs(L), fabs(H));
        double pad = 2.2e-16 * tn * 4.0 + 1e-300;
        bounds[0] = L - pad;
        bounds[1] = H + pad;
        bounds[2] = tn;
    }
}

// number of eigenvalues of T strictly below x (Sturm count of the LDL^T of T - xI)
__device__ int sturm_count(int n, const double *__restrict__ d, const double *__restrict__ e, double x,
                           double pivmin) {
    int cnt = 0;
    double q = d[0] - x;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0.0) cnt++;
    for (int i = 1; i < n; i++) {
        double ei = e[i - 1];
        q = d[i] - x - ei * ei / q;
        if (fabs(q) < pivmin) q = -pivmin;
        if (q < 0.0) cnt++;
    }
    return cnt;
}

__global__ void bisect_kernel(int n, const double *d, const double *e, const double *bounds, double *w) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double lo = bounds[0], hi = bounds[1];
    double tn = bounds[2];
    double pivmin = 1e-290 * fmax(1.0, tn * tn);
    for (int it = 0; it < 128; it++) {
        double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;
        if (hi - lo <= 2.0 * 2.2e-16 * fmax(fabs(lo), fabs(hi)) + 1e-300) break;
        int c = sturm_count(n, d, e, mid, pivmin);
        if (c <= j) lo = mid;
        else hi = mid;
    }
    w[j] = 0.5 * (lo + hi);
}

__device__ __forceinline__ double hash_unit(uint32_t a, uint32_t b) {
    uint32_t h = a * 0x9E3779B1u ^ (b + 0x7F4A7C15u) * 0x85EBCA77u;
    h ^= h >> 15;
    h *= 0x2C1B3C6Du;
    h ^= h >> 12;
    h *= 0x297A2D39u;
    h ^= h >> 15;
    return ((double)h / 4294967296.0) * 2.0 - 1.0;
}

// Inverse iteration, one thread per eigenvector; factorisation scratch laid out
// [array][row][vector] so that consecutive threads touch consecutive addresses.
__global__ void invit_kernel(int n, const double *__restrict__ d, const double *__restrict__ e,
                             const double *__restrict__ w, const double *__restrict__ bounds, int vlo, int nvec,
                             double *scr, double *z) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nvec) return;
    const double lam = w[vlo + t];
    const int64_t N = nvec;
    double *DL = scr, *DD = scr + (int64_t)n * N, *DU = scr + 2 * (int64_t)n * N, *DU2 = scr + 3 * (int64_t)n * N;
    unsigned char *PV = reinterpret_cast<unsigned char *>(scr + 4 * (int64_t)n * N);
#define IX(i) ((int64_t)(i) * N + t)
    const double tn = fmax(bounds[2], 1e-300);
    const double tiny = 2.2e-16 * tn;
    for (int i = 0; i < n; i++) {
        DD[IX(i)] = d[i] - lam;
        if (i < n - 1) {
            DL[IX(i)] = e[i];
            DU[IX(i)] = e[i];
        }
        if (i < n - 2) DU2[IX(i)] = 0.0;
    }
    // LU with partial pivoting (tridiagonal, fill-in in DU2)
    for (int i = 0; i < n - 1; i++) {
        double di = DD[IX(i)], li = DL[IX(i)];
        if (fabs(di) >= fabs(li)) {
            if (di == 0.0) di = tiny;
            DD[IX(i)] = di;
            double f = li / di;
            DL[IX(i)] = f;
            DD[IX(i + 1)] -= f * DU[IX(i)];
            PV[IX(i)] = 0;
        } else {
            double f = di / li;
            DD[IX(i)] = li;
            DL[IX(i)] = f;
            double tmp = DU[IX(i)];
            DU[IX(i)] = DD[IX(i + 1)];
            DD[IX(i + 1)] = tmp - f * DD[IX(i + 1)];
            if (i < n - 2) {
                DU2[IX(i)] = DU[IX(i + 1)];
                DU[IX(i + 1)] = -f * DU[IX(i + 1)];
            }
            PV[IX(i)] = 1;
        }
    }
    if (DD[IX(n - 1)] == 0.0) DD[IX(n - 1)] = tiny;
    for (int i = 0; i < n; i++) z[IX(i)] = hash_unit(i, vlo + t) + 0.5 * hash_unit(i + 7919, t + 104729);
    for (int it = 0; it < 3; it++) {
        // forward: apply L^-1 P
        for (int i = 0; i < n - 1; i++) {
            double bi = z[IX(i)], bn = z[IX(i + 1)];
            if (PV[IX(i)]) {
                z[IX(i)] = bn;
                z[IX(i + 1)] = bi - DL[IX(i)] * bn;
            } else {
                z[IX(i + 1)] = bn - DL[IX(i)] * bi;
            }
        }
        // back substitution with U (diag DD, super DU, second super DU2)
        double mx = 0.0;
        z[IX(n - 1)] /= DD[IX(n - 1)];
        if (n > 1) z[IX(n - 2)] = (z[IX(n - 2)] - DU[IX(n - 2)] * z[IX(n - 1)]) / DD[IX(n - 2)];
        for (int i = n - 3; i >= 0; i--)
            z[IX(i)] = (z[IX(i)] - DU[IX(i)] * z[IX(i + 1)] - DU2[IX(i)] * z[IX(i + 2)]) / DD[IX(i)];
        for (int i = 0; i < n; i++) mx = fmax(mx, fabs(z[IX(i)]));
        double inv = mx > 0.0 ? 1.0 / mx : 1.0;
        double s2 = 0.0;
        for (int i = 0; i < n; i++) {
            double v = z[IX(i)] * inv;
            z[IX(i)] = v;
            s2 += v * v;
        }
        double nrm = 1.0 / sqrt(s2);
        for (int i = 0; i < n; i++) z[IX(i)] *= nrm;
    }
#undef IX
}

// Modified Gram-Schmidt inside clusters of close eigenvalues (one block per cluster head)
__global__ void cluster_mgs_kernel(int n, const double *w, const double *bounds, int vlo, int nvec, double *z,
                                   double rel_tol) {
    __shared__ double sh[32];
    const int j = blockIdx.x;
    const double tol = rel_tol * fmax(bounds[2], 1e-300);
    if (j > 0 && w[vlo + j] - w[vlo + j - 1] <= tol) return;   // not a cluster head
    int len = 1;
    while (j + len < nvec && w[vlo + j + len] - w[vlo + j + len - 1] <= tol) len++;
    if (len == 1) return;
    const int64_t N = nvec;
    for (int c = 1; c < len; c++) {
        for (int pass = 0; pass < 2; pass++) {
            for (int p = 0; p < c; p++) {
                double s = 0.0;
                for (int i = threadIdx.x; i < n; i += blockDim.x) s += z[(int64_t)i * N + j + p] * z[(int64_t)i * N + j + c];
                s = block_sum(s, sh);
                for (int i = threadIdx.x; i < n; i += blockDim.x) z[(int64_t)i * N + j + c] -= s * z[(int64_t)i * N + j + p];
                __syncthreads();
            }
            double s2 = 0.0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) {
                double v = z[(int64_t)i * N + j + c];
                s2 += v * v;
            }
            s2 = block_sum(s2, sh);
            double inv = s2 > 0.0 ? 1.0 / sqrt(s2) : 0.0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) z[(int64_t)i * N + j + c] *= inv;
            __syncthreads();
        }
    }
}

// Z(:, c) = Q z(:, c) with Q = H_0 H_1 ... H_{n-2};  each block owns BT_COLS columns.
constexpr int BT_COLS = 4;
__global__ void backtransform_kernel(int n, const cplx *__restrict__ A, int64_t lda, const cplx *__restrict__ tau,
                                     const double *__restrict__ z, int nvec, cplx *Z, int64_t ldz) {
    __shared__ double sh[32];
    const int c0 = blockIdx.x * BT_COLS;
    const int nc = min(BT_COLS, nvec - c0);
    for (int c = 0; c < nc; c++)
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            Z[i + (int64_t)(c0 + c) * ldz] = mk(z[(int64_t)i * nvec + c0 + c], 0.0);
    __syncthreads();
    for (int k = n - 2; k >= 0; k--) {
        const cplx t = tau[k];
        if (t.x == 0.0 && t.y == 0.0) continue;
        const int m = n - k - 1;
        const cplx *v = A + (k + 1) + (int64_t)k * lda;
        double pr[BT_COLS], pi[BT_COLS];
#pragma unroll
        for (int c = 0; c < BT_COLS; c++) pr[c] = pi[c] = 0.0;
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            cplx vi = cconj(v[i]);
#pragma unroll
            for (int c = 0; c < BT_COLS; c++) {
                if (c < nc) {
                    cplx zz = Z[(k + 1 + i) + (int64_t)(c0 + c) * ldz];
                    cplx p = cmul(vi, zz);
                    pr[c] += p.x;
                    pi[c] += p.y;
                }
            }
        }
        cplx s[BT_COLS];
#pragma unroll
        for (int c = 0; c < BT_COLS; c++) {
            double a = block_sum(pr[c], sh);
            double b = block_sum(pi[c], sh);
            s[c] = cmul(t, mk(a, b));
        }
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            cplx vi = v[i];
#pragma unroll
            for (int c = 0; c < BT_COLS; c++) {
                if (c < nc) {
                    int64_t o = (k + 1 + i) + (int64_t)(c0 + c) * ldz;
                    Z[o] = csub(Z[o], cmul(vi, s[c]));
                }
            }
        }
        __syncthreads();
    }
}

struct HeevWork {
    double *d, *e, *bounds;
    cplx *tau, *ppart, *w;
};

static HeevWork heev_work(Context &c, int n) {
    HeevWork h;
    h.d = wsget<double>(c, "heev.d", n + 1);
    h.e = wsget<double>(c, "heev.e", n + 1);
    h.bounds = wsget<double>(c, "heev.bounds", 4);
    h.tau = wsget<cplx>(c, "heev.tau", n + 1);
    int nchunk = (n + HH_CHUNK - 1) / HH_CHUNK;
    h.ppart = wsget<cplx>(c, "heev.ppart", (size_t)nchunk * (n + 1));
    h.w = wsget<cplx>(c, "heev.w", n + 1);
    return h;
}

// Reduce A to tridiagonal form; d, e, tau in the named workspace, reflectors in A.
static void tridiag(Context &c, int n, cplx *A, int64_t lda, HeevWork &h) {
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

void heev(Context &c, int n, cplx *A, int64_t lda, double *w, int vlo, int vhi, cplx *Z, int64_t ldz) {
    if (n <= 0) return;
    FamScope fs(c, DCG_FAM_EIG, (16.0 / 3.0) * (double)n * n * n);
    HeevWork h = heev_work(c, n);
    {
        FamScope f1(c, DCG_FAM_EIG_TRI, (16.0 / 3.0) * (double)n * n * n);
        tridiag(c, n, A, lda, h);
    }
    {
        FamScope f2(c, DCG_FAM_EIG_VAL, (double)n * n);
        gersh_kernel<<<1, 1024, 0, c.stream>>>(n, h.d, h.e, h.bounds);
        DCG_LAUNCHED(c);
        bisect_kernel<<<grid1d(n, 128), 128, 0, c.stream>>>(n, h.d, h.e, h.bounds, w);
        DCG_LAUNCHED(c);
    }
    heev_vectors_only(c, n, A, lda, w, vlo, vhi, Z, ldz);
}

// Eigenvectors [vlo, vhi) of the matrix most recently reduced by heev() (its reflectors
// are still in A and its tridiagonal in the heev.* workspace).
void heev_vectors_only(Context &c, int n, cplx *A, int64_t lda, const double *w, int vlo, int vhi, cplx *Z,
                       int64_t ldz) {
    int nvec = vhi - vlo;
    if (nvec <= 0 || n <= 0) return;
    HeevWork h = heev_work(c, n);
    double *scr = wsget<double>(c, "heev.scr", (size_t)n * nvec * 5 + 16);
    double *zt = wsget<double>(c, "heev.z", (size_t)n * nvec + 16);
    FamScope fs(c, DCG_FAM_EIG, 8.0 * (double)n * n * nvec);
    {
        FamScope f3(c, DCG_FAM_EIG_VEC, 10.0 * (double)n * nvec);
        invit_kernel<<<grid1d(nvec, 64), 64, 0, c.stream>>>(n, h.d, h.e, w, h.bounds, vlo, nvec, scr, zt);
        DCG_LAUNCHED(c);
        cluster_mgs_kernel<<<nvec, 256, 0, c.stream>>>(n, w, h.bounds, vlo, nvec, zt, 1e-7);
        DCG_LAUNCHED(c);
    }
    FamScope f4(c, DCG_FAM_EIG_BACK, 8.0 * (double)n * n * nvec);
    backtransform_kernel<<<grid1d(nvec, BT_COLS), 256, 0, c.stream>>>(n, A, lda, h.tau, zt, nvec, Z, ldz);
    DCG_LAUNCHED(c);
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
