// E2 terms of a B' matrix from a band form instead of a tridiagonal form.
//
// The reference diagonalises B' (solve_A_subspace.F90:223 and its counterparts) only to evaluate,
// per outer index o,
//   e2o = -sum_m |(W^H v_o)_m|^2 / (alpha_o + w_m),   sco = sum_m |(W^H v_o)_m|^2 / (alpha_o + w_m)^2,
// which are -Re y^H (B' + alpha_o)^-1 y and |(B' + alpha_o)^-1 y|^2 for y = v_o in any unitary basis.
// Here B' = Q Bd Q^H with Bd Hermitian of lower bandwidth nb (stage one of a two-stage
// Hermitian reduction, as in LAPACK's ZHETRD_HE2HB: blocked Householder reflectors, each panel's
// trailing update a rank-2nb product), then one banded Gaussian elimination with partial
// pivoting per outer index on Bd + alpha_o (Golub & Van Loan, Matrix Computations, 4th ed.,
// 4.3.5: row interchanges widen the upper band of U to 2 nb).
//
// Against the one-stage reduction to tridiagonal form this trades one grid-wide synchronisation
// per column for a few launches per panel of nb columns: the panel QR runs in one CTA, the
// trailing updates are FP64 GEMMs over the whole GPU, and the per-index solves run one warp each.
#include "dcg_common.cuh"
#include "dcg_kernels.cuh"

namespace dcg {

// ------------------------------------------------------------------------- panel QR
// Householder QR of the panel P (m x nb, column-major, ldp) with r = min(nb, m - 1) reflectors
// H_j = I - tau_j v_j v_j^H (ZLARFG convention: H_j^H x = beta e_1, beta real), applied as
// Q^H P with Q = H_0 H_1 ... H_{r-1} = I - V T V^H.  Outputs: P overwritten by Q^H P (upper
// triangle in its first r rows, zeros below); V (m x r, ldv = m, unit lower trapezoidal with
// explicit ones and zeros), also copied to V2 when V2 is not null; T (r x r upper triangular,
// ldt).  One CTA; warp w owns panel column w for the dots and updates; v_j staged in shared
// memory.
constexpr int kBandThreads = 512;
constexpr int kBandMaxR = 32;   // reflectors per panel the kernel holds (nb <= kBandMaxR)

__global__ void __launch_bounds__(kBandThreads) band_panel_qr_kernel(int m, int nb, int r, cplx *P, int64_t ldp,
                                                                    cplx *V, cplx *V2, cplx *T, int ldt) {
    extern __shared__ cplx bsm[];
    cplx *sv = bsm;                       // v_j, m entries
    __shared__ double red[2][32];
    __shared__ cplx s_tau[kBandMaxR];
    __shared__ cplx s_G[kBandMaxR * kBandMaxR];   // G(i, j) = v_i^H v_j, i < j
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int j = 0; j < r; j++) {
        cplx *x = P + j + (int64_t)j * ldp;   // x[0] = alpha, x[1 .. m-j-1]
        const int len = m - j;
        double ss = 0.0;
        for (int i = 1 + threadIdx.x; i < len; i += blockDim.x) ss += cabs2(x[i]);
        for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
        if (lane == 0) red[0][warp] = ss;
        __syncthreads();
        double xs = 0.0;
        for (int w = 0; w < nw; w++) xs += red[0][w];   // same order in every thread
        const cplx alpha = x[0];
        cplx tau, scale;
        double beta;
        if (xs == 0.0 && alpha.y == 0.0) {   // nothing to annihilate: H_j = I
            tau = mk(0.0, 0.0);
            beta = alpha.x;
            scale = mk(0.0, 0.0);
        } else {
            const double nrm = sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xs);
            beta = alpha.x >= 0.0 ? -nrm : nrm;
            tau = mk((beta - alpha.x) / beta, -alpha.y / beta);
            scale = cdiv(mk(1.0, 0.0), mk(alpha.x - beta, alpha.y));
        }
        // v_j = [1; x[1:] * scale] into shared memory and V (and V2); P column j -> beta e_1
        for (int i = threadIdx.x; i < m; i += blockDim.x) {
            cplx v;
            if (i < j) v = mk(0.0, 0.0);
            else if (i == j) v = mk(1.0, 0.0);
            else v = (tau.x == 0.0 && tau.y == 0.0) ? mk(0.0, 0.0) : cmul(x[i - j], scale);
            sv[i] = v;
            V[i + (int64_t)j * m] = v;
            if (V2) V2[i + (int64_t)j * m] = v;
        }
        __syncthreads();
        if (threadIdx.x == 0) s_tau[j] = tau;
        for (int i = threadIdx.x; i < len; i += blockDim.x) x[i] = i == 0 ? mk(beta, 0.0) : mk(0.0, 0.0);
        // columns c > j of the panel: c -= conj(tau) v (v^H c)
        if (tau.x != 0.0 || tau.y != 0.0) {
            for (int cidx = j + 1 + warp; cidx < nb; cidx += nw) {
                cplx *col = P + (int64_t)cidx * ldp;
                double dr = 0.0, di = 0.0;
                for (int i = j + lane; i < m; i += 32) {
                    const cplx v = sv[i], a = col[i];
                    dr = fma(v.x, a.x, fma(v.y, a.y, dr));   // conj(v) a
                    di = fma(v.x, a.y, fma(-v.y, a.x, di));
                }
                for (int o = 16; o > 0; o >>= 1) {
                    dr += __shfl_xor_sync(0xffffffffu, dr, o);
                    di += __shfl_xor_sync(0xffffffffu, di, o);
                }
                const cplx f = cmul(cconj(tau), mk(dr, di));
                for (int i = j + lane; i < m; i += 32) col[i] = csub(col[i], cmul(sv[i], f));
            }
        }
        __syncthreads();
    }
    // T (ZLARFT, forward, columnwise): T(j,j) = tau_j, T(0:j, j) = -tau_j T(0:j,0:j) G(0:j, j)
    for (int p = warp; p < r * r; p += nw) {
        const int i = p % r, j = p / r;
        if (i >= j) continue;
        const cplx *vi = V + (int64_t)i * m, *vj = V + (int64_t)j * m;
        double gr = 0.0, gi = 0.0;
        for (int q = j + lane; q < m; q += 32) {   // v_j is zero above row j
            const cplx a = vi[q], b = vj[q];
            gr = fma(a.x, b.x, fma(a.y, b.y, gr));
            gi = fma(a.x, b.y, fma(-a.y, b.x, gi));
        }
        for (int o = 16; o > 0; o >>= 1) {
            gr += __shfl_xor_sync(0xffffffffu, gr, o);
            gi += __shfl_xor_sync(0xffffffffu, gi, o);
        }
        if (lane == 0) s_G[i + kBandMaxR * j] = mk(gr, gi);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int j = 0; j < r; j++) {
            const cplx tj = s_tau[j];
            for (int i = 0; i < j; i++) {   // (T(0:j,0:j) G(0:j, j))_i, T upper triangular
                cplx acc = mk(0.0, 0.0);
                for (int q = i; q < j; q++) acc = cadd(acc, cmul(T[i + (int64_t)q * ldt], s_G[q + kBandMaxR * j]));
                T[i + (int64_t)j * ldt] = cmul(mk(-tj.x, -tj.y), acc);
            }
            T[j + (int64_t)j * ldt] = tj;
            for (int i = j + 1; i < r; i++) T[i + (int64_t)j * ldt] = mk(0.0, 0.0);
        }
    }
}

// ------------------------------------------------------------------------- banded solves
// Per outer index o (one warp): Gaussian elimination with partial pivoting on Bd + alpha_o,
// Bd the Hermitian band matrix held in the lower band of A (A(i, j), 0 <= i - j <= NB; the upper
// band is its conjugate), right-hand side y_o = Y[:, o]; then back substitution with
//   e2o = -Re y^H x,  sco = |x|^2.
// Row interchanges widen the upper band of U to 2 NB, so the active rows i .. i+NB live in a
// shared-memory window of NB+1 rows by 2NB+1 columns (columns i .. i+2NB), both indexed
// cyclically (row q in slot q % (NB+1), column q in slot q % (2NB+1)).  Each finished row of U
// (its right-hand side in place of the pivot, which goes to a separate array) is written to
// scratch for the back substitution: Us holds nouter * n rows of 2NB+1 entries, then nouter * n
// pivots.
template <int NB>
__global__ void __launch_bounds__(64) band_solve_e2_kernel(int n, const cplx *__restrict__ A, int64_t lda,
                                                          const cplx *__restrict__ Y, int64_t ldy, int nouter,
                                                          const double *__restrict__ alpha, cplx *Us, double *e2o,
                                                          double *sco) {
    constexpr int R = NB + 1, C = 2 * NB + 1, CPL = (C + 31) / 32;
    __shared__ cplx win[2][R][C];
    __shared__ cplx rhs[2][R];
    __shared__ cplx xs[2][C];
    const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
    const int o = blockIdx.x * 2 + wl;
    if (o >= nouter) return;   // whole warp; no block-level barrier below
    cplx(*W)[C] = win[wl];
    cplx *b = rhs[wl];
    const double al = alpha[o];
    const cplx *y = Y + (int64_t)o * ldy;
    cplx *U = Us + (int64_t)o * n * C;
    cplx *pivs = Us + (int64_t)nouter * n * C + (int64_t)o * n;
    // element (row, col) of Bd + alpha I from the lower band
    auto band = [&](int row, int col) -> cplx {
        if (row >= n || col >= n) return mk(0.0, 0.0);
        const int d = row - col;
        if (d > NB || d < -NB) return mk(0.0, 0.0);
        cplx v = d >= 0 ? A[row + (int64_t)col * lda] : cconj(A[col + (int64_t)row * lda]);
        if (d == 0) v = mk(v.x + al, 0.0);
        return v;
    };
    for (int rr = 0; rr < R; rr++) {
        for (int cc = lane; cc < C; cc += 32) W[rr][cc] = band(rr, cc);
        if (lane == 0) b[rr] = rr < n ? y[rr] : mk(0.0, 0.0);
    }
    __syncwarp();
    for (int i = 0; i < n; i++) {
        const int s0 = i % R, c0 = i % C;
        const int rows = min(NB, n - 1 - i);   // rows below the pivot row
        // pivot: largest |entry| of column i over rows i .. i + rows, the first on ties
        double best = -1.0;
        int bi = 0;
        if (lane <= rows) {
            best = cabs2(W[(i + lane) % R][c0]);
            bi = lane;
        }
        for (int off = 16; off > 0; off >>= 1) {
            const double ob = __shfl_xor_sync(0xffffffffu, best, off);
            const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
            if (ob > best || (ob == best && oi < bi)) {
                best = ob;
                bi = oi;
            }
        }
        if (bi != 0) {
            const int sp = (i + bi) % R;
            for (int cc = lane; cc < C; cc += 32) {
                const cplx t = W[s0][cc];
                W[s0][cc] = W[sp][cc];
                W[sp][cc] = t;
            }
            if (lane == 0) {
                const cplx t = b[s0];
                b[s0] = b[sp];
                b[sp] = t;
            }
        }
        __syncwarp();
        const cplx piv = W[s0][c0];
        const cplx ipiv = cdiv(mk(1.0, 0.0), piv);
        cplx prow[CPL];
#pragma unroll
        for (int q = 0; q < CPL; q++) {
            const int cc = lane + 32 * q;
            prow[q] = cc < C ? W[s0][(c0 + cc) % C] : mk(0.0, 0.0);
        }
        const cplx bp = b[s0];
        __syncwarp();
        // eliminate column i from rows i+1 .. i+rows (columns i+1 .. i+2NB)
        for (int rr = 1; rr <= rows; rr++) {
            const int sr = (i + rr) % R;
            const cplx f = cmul(W[sr][c0], ipiv);
#pragma unroll
            for (int q = 0; q < CPL; q++) {
                const int cc = lane + 32 * q;
                if (cc >= 1 && cc < C) {
                    const int sl = (c0 + cc) % C;
                    W[sr][sl] = csub(W[sr][sl], cmul(f, prow[q]));
                }
            }
            if (lane == 0) b[sr] = csub(b[sr], cmul(f, bp));
        }
        // U row i: right-hand side in entry 0, U(i, i+cc) in entry cc; the pivot apart
#pragma unroll
        for (int q = 0; q < CPL; q++) {
            const int cc = lane + 32 * q;
            if (cc < C) U[(int64_t)i * C + cc] = cc == 0 ? bp : prow[q];
        }
        if (lane == 0) pivs[i] = piv;
        __syncwarp();
        // column slot c0 now serves column i + C (zero in rows i+1 .. i+NB: their entries reach
        // column i + 2NB at most); row slot s0 serves row i + R, which enters with its band
        for (int rr = 1 + lane; rr <= NB; rr += 32) W[(i + rr) % R][c0] = mk(0.0, 0.0);
        const int nr = i + R;
        for (int cc = lane; cc < C; cc += 32) {
            const int col = i + 1 + cc;
            W[s0][col % C] = band(nr, col);
        }
        if (lane == 0) b[s0] = nr < n ? y[nr] : mk(0.0, 0.0);
        __syncwarp();
    }
    // back substitution: x_i = (b_i - sum_{c=1}^{2NB} U(i, i+c) x_{i+c}) / u_ii, x kept cyclically
    cplx *xw = xs[wl];
    for (int cc = lane; cc < C; cc += 32) xw[cc] = mk(0.0, 0.0);
    __syncwarp();
    double er = 0.0, sc = 0.0;
    for (int i = n - 1; i >= 0; i--) {
        double sr = 0.0, si = 0.0;
        for (int cc = 1 + lane; cc < C; cc += 32) {
            const int col = i + cc;
            if (col >= n) continue;
            const cplx u = U[(int64_t)i * C + cc], xv = xw[col % C];
            sr = fma(u.x, xv.x, fma(-u.y, xv.y, sr));
            si = fma(u.x, xv.y, fma(u.y, xv.x, si));
        }
        for (int off = 16; off > 0; off >>= 1) {
            sr += __shfl_xor_sync(0xffffffffu, sr, off);
            si += __shfl_xor_sync(0xffffffffu, si, off);
        }
        const cplx bi = U[(int64_t)i * C];
        const cplx xi = cdiv(mk(bi.x - sr, bi.y - si), pivs[i]);
        __syncwarp();
        if (lane == 0) xw[i % C] = xi;
        __syncwarp();
        const cplx yi = y[i];
        er = fma(yi.x, xi.x, fma(yi.y, xi.y, er));   // Re conj(y) x
        sc = fma(xi.x, xi.x, fma(xi.y, xi.y, sc));
    }
    if (lane == 0) {
        e2o[o] = -er;
        sco[o] = sc;
    }
}

// ------------------------------------------------------------------------- driver
bool band_e2_pays(int n, int nouter) {
    const char *e = getenv("DCG_BPRIME_ROUTE");   // "band" / "tridiag": force one route (read per call)
    const int force = !e ? 0 : (std::string(e) == "band" ? 1 : (std::string(e) == "tridiag" ? -1 : 0));
    // Off unless forced: measured at 20/12/300 (B' of about 700 rows for A and C) the band route
    // took the A/C stage from 63 to 195 ms.  Its panel QR runs in one CTA, bound by one SM's FP64
    // rate (about two FMAs per clock) and by L2 latency, 43 panels per matrix, and its
    // tall-skinny trailing products fill few SMs; the one-stage reduction spreads all of its
    // work over the GPU and overlaps the two matrices in one launch.
    (void)kBandMinN;
    return force > 0 && n > kBandNB + 1 && nouter > 0;
}

void band_e2(Context &c, int slot, int n, cplx *A, int64_t lda, const cplx *VC, int64_t ldvc, int nouter,
             const double *alpha, double *e2o, double *sco) {
    if (n <= 0 || nouter <= 0) return;
    constexpr int nb = kBandNB;
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0), mone = mk(-1.0, 0.0), mhalf = mk(-0.5, 0.0);
    auto nm = [slot](const char *b) { return std::string(b) + "#" + std::to_string(slot); };
    FamScope fs(c, DCG_FAM_EIG, (16.0 / 3.0) * (double)n * n * n);
    cplx *Y = wsget<cplx>(c, nm("band.Y"), (size_t)n * nouter);
    DCG_CUDA(cudaMemcpy2DAsync(Y, sizeof(cplx) * n, VC, sizeof(cplx) * ldvc, sizeof(cplx) * n, nouter,
                               cudaMemcpyDeviceToDevice, c.stream));
    {
        FamScope ft(c, DCG_FAM_EIG_TRI, (16.0 / 3.0) * (double)n * n * n);
        const int mmax = std::max(1, n - nb);
        cplx *PVX = wsget<cplx>(c, nm("band.PVX"), (size_t)mmax * 3 * nb);   // [V | X | V]
        cplx *VT = wsget<cplx>(c, nm("band.VT"), (size_t)mmax * nb);
        cplx *T = wsget<cplx>(c, nm("band.T"), (size_t)nb * nb);
        cplx *S = wsget<cplx>(c, nm("band.S"), (size_t)nb * nb);
        cplx *Um = wsget<cplx>(c, nm("band.U"), (size_t)nb * nb);
        cplx *Z = wsget<cplx>(c, nm("band.Z"), (size_t)nb * nouter);
        cplx *Z2 = wsget<cplx>(c, nm("band.Z2"), (size_t)nb * nouter);
        const size_t smem = sizeof(cplx) * (size_t)mmax;
        if (smem > 48 * 1024)
            DCG_CUDA(cudaFuncSetAttribute(band_panel_qr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)smem));
        for (int k = 0; k + nb < n; k += nb) {
            const int m = n - k - nb;
            const int r = std::min(nb, m - 1);
            if (r <= 0) break;
            cplx *P = A + (k + nb) + (int64_t)k * lda;
            cplx *V = PVX, *X = PVX + (size_t)r * m, *V2 = PVX + (size_t)2 * r * m;
            band_panel_qr_kernel<<<1, kBandThreads, sizeof(cplx) * m, c.stream>>>(m, nb, r, P, lda, V, V2, T, nb);
            DCG_LAUNCHED(c);
            cplx *A22 = A + (k + nb) + (int64_t)(k + nb) * lda;
            // X = A22 V T;  X -= 1/2 V (T^H V^H X);  A22 -= V X^H + X V^H  (A22 <- Q^H A22 Q)
            zgemm(c, OP_N, OP_N, m, r, r, one, V, m, 0, T, nb, 0, zero, VT, m, 0);
            zgemm(c, OP_N, OP_N, m, r, m, one, A22, lda, 0, VT, m, 0, zero, X, m, 0);
            zgemm(c, OP_C, OP_N, r, r, m, one, V, m, 0, X, m, 0, zero, S, nb, 0);
            zgemm(c, OP_C, OP_N, r, r, r, one, T, nb, 0, S, nb, 0, zero, Um, nb, 0);
            zgemm(c, OP_N, OP_N, m, r, r, mhalf, V, m, 0, Um, nb, 0, one, X, m, 0);
            zgemm(c, OP_N, OP_C, m, m, 2 * r, mone, PVX, m, 0, X, m, 0, one, A22, lda, 0);
            // Y(k+nb:, :) <- Q^H Y(k+nb:, :) = Y - V T^H (V^H Y)
            cplx *Y2 = Y + (k + nb);
            zgemm(c, OP_C, OP_N, r, nouter, m, one, V, m, 0, Y2, n, 0, zero, Z, nb, 0);
            zgemm(c, OP_C, OP_N, r, nouter, r, one, T, nb, 0, Z, nb, 0, zero, Z2, nb, 0);
            zgemm(c, OP_N, OP_N, m, nouter, r, mone, V, m, 0, Z2, nb, 0, one, Y2, n, 0);
        }
    }
    constexpr int C = 2 * nb + 1;
    cplx *Us = wsget<cplx>(c, nm("band.Us"), (size_t)nouter * n * C + (size_t)nouter * n);
    band_solve_e2_kernel<nb><<<(unsigned)((nouter + 1) / 2), 64, 0, c.stream>>>(n, A, lda, Y, n, nouter, alpha, Us,
                                                                                 e2o, sco);
    DCG_LAUNCHED(c);
}

}  // namespace dcg
