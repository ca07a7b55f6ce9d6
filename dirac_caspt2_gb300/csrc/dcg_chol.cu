// Blocked Cholesky factorisation A = L L^H of a Hermitian matrix and the solve A X = B on the
// device (Golub & Van Loan, Matrix Computations, 4th ed., 4.2.8-4.2.9: right-looking block
// form).  Per 48-column panel: the diagonal block is factored in one block's shared memory,
// the rows below it by a triangular solve against it, and the trailing matrix by one FP64
// GEMM.  The factorisation records the first non-positive pivot (the matrix is then not
// positive definite).
#include "dcg_common.cuh"

namespace dcg {

namespace {

constexpr int CH_NB = 48;   // panel width: the 48 x 49 complex tile fits the 48 KB of static shared memory

// Factor the kb x kb diagonal block at A (lower triangle read and written), in shared memory.
// info: the first failing global pivot index + 1 (0 keeps going; a set info skips the work).
__global__ void __launch_bounds__(256) chol_panel_kernel(int kb, int k0, cplx *A, int64_t lda, int *info) {
    __shared__ cplx s[CH_NB][CH_NB + 1];
    __shared__ int bad;
    if (*info != 0) return;
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        const int i = e % kb, j = e / kb;
        s[i][j] = A[i + (int64_t)j * lda];
    }
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    for (int j = 0; j < kb; j++) {
        const double piv = s[j][j].x;
        if (!(piv > 0.0)) {   // also catches NaN
            if (threadIdx.x == 0) bad = k0 + j + 1;
            __syncthreads();
            break;
        }
        const double r = sqrt(piv), inv = 1.0 / r;
        __syncthreads();
        for (int i = j + 1 + threadIdx.x; i < kb; i += blockDim.x) s[i][j] = mk(s[i][j].x * inv, s[i][j].y * inv);
        if (threadIdx.x == 0) s[j][j] = mk(r, 0.0);
        __syncthreads();
        // trailing lower part: s[i][l] -= s[i][j] conj(s[l][j]), j < l <= i
        const int m = kb - j - 1;
        for (int e = threadIdx.x; e < m * m; e += blockDim.x) {
            const int i = j + 1 + e % m, l = j + 1 + e / m;
            if (l <= i) s[i][l] = csub(s[i][l], cmul(s[i][j], cconj(s[l][j])));
        }
        __syncthreads();
    }
    if (bad) {
        if (threadIdx.x == 0) *info = bad;
        return;
    }
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        const int i = e % kb, j = e / kb;
        if (i >= j) A[i + (int64_t)j * lda] = s[i][j];
    }
}

// Rows below the panel: X L11^H = A21, row by row (one thread per row, L11 in shared memory).
__global__ void __launch_bounds__(128) chol_trsm_rows_kernel(int m, int kb, const cplx *L11, cplx *A21, int64_t lda,
                                                              const int *info) {
    __shared__ cplx l[CH_NB][CH_NB + 1];
    if (*info != 0) return;
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        const int i = e % kb, j = e / kb;
        l[i][j] = (i >= j) ? L11[i + (int64_t)j * lda] : mk(0.0, 0.0);
    }
    __syncthreads();
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= m) return;
    cplx x[CH_NB];
#pragma unroll 4
    for (int j = 0; j < kb; j++) {
        cplx a = A21[r + (int64_t)j * lda];
        for (int i = 0; i < j; i++) a = csub(a, cmul(x[i], cconj(l[j][i])));
        const double inv = 1.0 / l[j][j].x;
        x[j] = mk(a.x * inv, a.y * inv);
    }
    for (int j = 0; j < kb; j++) A21[r + (int64_t)j * lda] = x[j];
}

// Forward (lower = true: L11 Y = B) or backward (L11^H X = B) triangular solve of a kb-row slab
// of B (kb x nrhs, ldb), one thread per right-hand side.
__global__ void __launch_bounds__(128) chol_trsv_cols_kernel(int kb, int nrhs, const cplx *L11, int64_t lda, cplx *B,
                                                              int64_t ldb, bool lower) {
    __shared__ cplx l[CH_NB][CH_NB + 1];
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        const int i = e % kb, j = e / kb;
        l[i][j] = (i >= j) ? L11[i + (int64_t)j * lda] : mk(0.0, 0.0);
    }
    __syncthreads();
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nrhs) return;
    cplx *b = B + (int64_t)q * ldb;
    cplx x[CH_NB];
    if (lower) {
        for (int i = 0; i < kb; i++) {
            cplx a = b[i];
            for (int j = 0; j < i; j++) a = csub(a, cmul(l[i][j], x[j]));
            const double inv = 1.0 / l[i][i].x;
            x[i] = mk(a.x * inv, a.y * inv);
        }
    } else {   // L11^H x = b: row i of L11^H is conj(column i of L11)
        for (int i = kb - 1; i >= 0; i--) {
            cplx a = b[i];
            for (int j = i + 1; j < kb; j++) a = csub(a, cmul(cconj(l[j][i]), x[j]));
            const double inv = 1.0 / l[i][i].x;
            x[i] = mk(a.x * inv, a.y * inv);
        }
    }
    for (int i = 0; i < kb; i++) b[i] = x[i];
}

}  // namespace

void zpotrf_lower(Context &c, int n, cplx *A, int64_t lda, int *info) {
    DCG_CUDA(cudaMemsetAsync(info, 0, sizeof(int), c.stream));
    const cplx mone = mk(-1.0, 0.0), one = mk(1.0, 0.0);
    for (int k0 = 0; k0 < n; k0 += CH_NB) {
        const int kb = std::min(CH_NB, n - k0);
        cplx *A11 = A + k0 + (int64_t)k0 * lda;
        chol_panel_kernel<<<1, 256, 0, c.stream>>>(kb, k0, A11, lda, info);
        DCG_LAUNCHED(c);
        const int m = n - k0 - kb;
        if (m <= 0) break;
        cplx *A21 = A11 + kb;
        chol_trsm_rows_kernel<<<grid1d(m, 128), 128, 0, c.stream>>>(m, kb, A11, A21, lda, info);
        DCG_LAUNCHED(c);
        // A22 -= A21 A21^H (full square: the upper part is ignored by the later panels)
        cplx *A22 = A21 + (int64_t)kb * lda;
        zgemm(c, OP_N, OP_C, m, m, kb, mone, A21, lda, 0, A21, lda, 0, one, A22, lda, 0, 1);
    }
}

void zpotrs_lower(Context &c, int n, const cplx *L, int64_t lda, cplx *B, int64_t ldb, int nrhs) {
    if (n <= 0 || nrhs <= 0) return;
    const cplx mone = mk(-1.0, 0.0), one = mk(1.0, 0.0);
    const unsigned g = grid1d(nrhs, 128);
    for (int k0 = 0; k0 < n; k0 += CH_NB) {   // L Y = B
        const int kb = std::min(CH_NB, n - k0);
        const cplx *L11 = L + k0 + (int64_t)k0 * lda;
        chol_trsv_cols_kernel<<<g, 128, 0, c.stream>>>(kb, nrhs, L11, lda, B + k0, ldb, true);
        DCG_LAUNCHED(c);
        const int m = n - k0 - kb;
        if (m > 0) zgemm(c, OP_N, OP_N, m, nrhs, kb, mone, L11 + kb, lda, 0, B + k0, ldb, 0, one, B + k0 + kb, ldb, 0, 1);
    }
    for (int k0 = ((n - 1) / CH_NB) * CH_NB; k0 >= 0; k0 -= CH_NB) {   // L^H X = Y
        const int kb = std::min(CH_NB, n - k0);
        const cplx *L11 = L + k0 + (int64_t)k0 * lda;
        const int m = n - k0 - kb;
        if (m > 0) zgemm(c, OP_C, OP_N, kb, nrhs, m, mone, L11 + kb, lda, 0, B + k0 + kb, ldb, 0, one, B + k0, ldb, 0, 1);
        chol_trsv_cols_kernel<<<g, 128, 0, c.stream>>>(kb, nrhs, L11, lda, B + k0, ldb, false);
        DCG_LAUNCHED(c);
    }
}

}  // namespace dcg

namespace dcg {

namespace {

__device__ __forceinline__ double wsum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Wm[m + Mp i] = 1 / (D_m + alpha_i) (complex, zero imaginary part); A = U o Wm.
__global__ void wb_weights_kernel(int Mp, int nouter, const double *__restrict__ Dd, const double *__restrict__ alpha,
                                  const cplx *__restrict__ U, int64_t ldu, cplx *Wm, cplx *A) {
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)Mp * nouter) return;
    const int m = (int)(e % Mp), i = (int)(e / Mp);
    const double w = 1.0 / (Dd[m] + alpha[i]);
    Wm[e] = mk(w, 0.0);
    const cplx u = U[m + ldu * i];
    A[e] = mk(u.x * w, u.y * w);
}

// Phi[p + npair m] = conj(Ps[m, k]) Ps[m, l] for the packed pairs p = (k <= l) of r columns.
__global__ void wb_phi_kernel(int Mp, int r, const cplx *__restrict__ Ps, int64_t ldp, cplx *Phi) {
    const int npair = r * (r + 1) / 2;
    const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (int64_t)npair * Mp) return;
    const int p = (int)(e % npair), m = (int)(e / npair);
    int q = p, k = 0;
    while (q >= r - k) {
        q -= r - k;
        k++;
    }
    const int l = k + q;
    Phi[e] = cmul(cconj(Ps[m + ldp * k]), Ps[m + ldp * l]);
}

// Per outer index i (one block): C_i (r x r Hermitian, unpacked from column i of Cp into shared
// memory) x = b_i by Gaussian elimination with partial pivoting (rows updated in parallel);
// x to X[:, i].
__global__ void __launch_bounds__(256) wb_solve_kernel(int r, const cplx *__restrict__ Cp, const cplx *__restrict__ Bv,
                                                       cplx *X) {
    extern __shared__ double2 wsm[];
    cplx *C = wsm, *xv = C + r * r;
    __shared__ int piv_s;
    const int i = blockIdx.x, npair = r * (r + 1) / 2;
    const cplx *cp = Cp + (int64_t)npair * i;
    for (int p = threadIdx.x; p < npair; p += blockDim.x) {
        int q = p, k = 0;
        while (q >= r - k) {
            q -= r - k;
            k++;
        }
        const int l = k + q;
        const cplx v = cp[p];
        C[k + r * l] = v;
        C[l + r * k] = cconj(v);
    }
    for (int k = threadIdx.x; k < r; k += blockDim.x) xv[k] = Bv[k + (int64_t)r * i];
    __syncthreads();
    for (int k = 0; k < r; k++) {
        if (threadIdx.x == 0) {
            int p = k;
            double best = cabs2(C[k + r * k]);
            for (int q = k + 1; q < r; q++) {
                const double v = cabs2(C[q + r * k]);
                if (v > best) {
                    best = v;
                    p = q;
                }
            }
            piv_s = p;
        }
        __syncthreads();
        const int p = piv_s;
        if (p != k) {
            for (int j = threadIdx.x; j < r; j += blockDim.x) {
                const cplx t = C[k + r * j];
                C[k + r * j] = C[p + r * j];
                C[p + r * j] = t;
            }
            if (threadIdx.x == 0) {
                const cplx t = xv[k];
                xv[k] = xv[p];
                xv[p] = t;
            }
        }
        __syncthreads();
        const cplx inv = cdiv(mk(1.0, 0.0), C[k + r * k]);
        for (int q = k + 1 + threadIdx.x; q < r; q += blockDim.x) {
            const cplx f = cmul(C[q + r * k], inv);
            for (int j = k + 1; j < r; j++) C[q + r * j] = csub(C[q + r * j], cmul(f, C[k + r * j]));
            xv[q] = csub(xv[q], cmul(f, xv[k]));
        }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int k = r - 1; k >= 0; k--) {
            cplx s = xv[k];
            for (int j = k + 1; j < r; j++) s = csub(s, cmul(C[k + r * j], xv[j]));
            xv[k] = cdiv(s, C[k + r * k]);
        }
    __syncthreads();
    for (int k = threadIdx.x; k < r; k += blockDim.x) X[k + (int64_t)r * i] = xv[k];
}

// Per outer index i: z = Wm o Zm; e2o = -Re u^H z, sco = |z|^2 (fixed-order block reduction).
__global__ void __launch_bounds__(256) wb_e2_kernel(int Mp, const cplx *__restrict__ U, int64_t ldu,
                                                    const cplx *__restrict__ Zm, const cplx *__restrict__ Wm,
                                                    double *e2o, double *sco) {
    __shared__ double red[2][8];
    const int i = blockIdx.x, lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double e = 0.0, s2 = 0.0;
    for (int m = threadIdx.x; m < Mp; m += blockDim.x) {
        const double w = Wm[m + (int64_t)Mp * i].x;
        const cplx zz = Zm[m + (int64_t)Mp * i];
        const cplx z = mk(zz.x * w, zz.y * w), u = U[m + ldu * i];
        e += u.x * z.x + u.y * z.y;
        s2 += z.x * z.x + z.y * z.y;
    }
    e = wsum(e);
    s2 = wsum(s2);
    if (lane == 0) {
        red[0][warp] = e;
        red[1][warp] = s2;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double te = 0.0, ts = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            te += red[0][w];
            ts += red[1][w];
        }
        e2o[i] = -te;
        sco[i] = ts;
    }
}

}  // namespace

// With M_i = D + alpha_i (diagonal over the Mp determinants), the compression of M_i to the
// orthogonal complement of the r orthonormal columns of Ps has, on that complement, the inverse
// M^-1 - M^-1 Ps C^-1 Ps^H M^-1 with C = Ps^H M^-1 Ps (r x r).  For u = U[:, i] in the
// complement: z = M^-1 (u - Ps C^-1 b) with b = Ps^H M^-1 u, and e2o = -Re u^H z,
// sco = |z|^2.  The r x r matrices of all outer indices come from one GEMM of the packed pair
// products of Ps with the weights 1 / (D + alpha); then one pivoted r x r solve per index.
void launch_woodbury_e2(Context &c, int Mp, int r, const cplx *U, int64_t ldu, const cplx *Ps, int64_t ldp,
                        const double *Dd, const double *alpha, int nouter, double *e2o, double *sco) {
    if (nouter <= 0) return;
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0), mone = mk(-1.0, 0.0);
    const int npair = r * (r + 1) / 2;
    const size_t mo = (size_t)Mp * nouter;
    constexpr int kWbMaxR = 112;   // (r^2 + r) complex in one block's shared memory
    cplx *Wm = wsget<cplx>(c, "wb.W", mo);
    cplx *A = wsget<cplx>(c, "wb.A", mo);
    cplx *Phi = wsget<cplx>(c, "wb.Phi", (size_t)npair * Mp);
    cplx *Cp = wsget<cplx>(c, "wb.C", (size_t)npair * nouter);
    cplx *Bv = wsget<cplx>(c, "wb.B", (size_t)r * nouter);
    cplx *X = wsget<cplx>(c, "wb.X", (size_t)r * nouter);
    cplx *Zm = wsget<cplx>(c, "wb.Z", mo);
    wb_weights_kernel<<<grid1d((int64_t)mo, 256), 256, 0, c.stream>>>(Mp, nouter, Dd, alpha, U, ldu, Wm, A);
    DCG_LAUNCHED(c);
    wb_phi_kernel<<<grid1d((int64_t)npair * Mp, 256), 256, 0, c.stream>>>(Mp, r, Ps, ldp, Phi);
    DCG_LAUNCHED(c);
    // C_i, packed: r(r+1)/2 x nouter x Mp, the largest product of the route.  On the split
    // path it runs on the tensor cores (C_i enters a well-conditioned r x r solve, not the
    // metric's inverse).
    if (c.precision == DCG_PREC_SPLIT && npair >= 128)
        zgemm_split(c, npair, nouter, Mp, 1, Phi, 1, npair, 0, Wm, Mp, 0, Cp, 1, npair, 0, false, c.split_lbo,
                    c.split_sbo);
    else
        zgemm(c, OP_N, OP_N, npair, nouter, Mp, one, Phi, npair, 0, Wm, Mp, 0, zero, Cp, npair, 0, 1);
    zgemm(c, OP_C, OP_N, r, nouter, Mp, one, Ps, ldp, 0, A, Mp, 0, zero, Bv, r, 0, 1);            // b_i
    if (r > kWbMaxR) throw Error{DCG_E_ARG, "deflated Gram route: more eigenvalues under the cutoff than it takes"};
    const size_t smem = sizeof(cplx) * ((size_t)r * r + (size_t)r);
    DCG_CUDA(cudaFuncSetAttribute(wb_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    wb_solve_kernel<<<nouter, 256, smem, c.stream>>>(r, Cp, Bv, X);
    DCG_LAUNCHED(c);
    DCG_CUDA(cudaMemcpy2DAsync(Zm, (size_t)Mp * sizeof(cplx), U, (size_t)ldu * sizeof(cplx), (size_t)Mp * sizeof(cplx),
                               nouter, cudaMemcpyDeviceToDevice, c.stream));
    zgemm(c, OP_N, OP_N, Mp, nouter, r, mone, Ps, ldp, 0, X, r, 0, one, Zm, Mp, 0, 1);               // u - Ps x
    wb_e2_kernel<<<nouter, 256, 0, c.stream>>>(Mp, U, ldu, Zm, Wm, e2o, sco);
    DCG_LAUNCHED(c);
}

}  // namespace dcg
