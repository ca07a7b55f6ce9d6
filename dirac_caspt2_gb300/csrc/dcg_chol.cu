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
