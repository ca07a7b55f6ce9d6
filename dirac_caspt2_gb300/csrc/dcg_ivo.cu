// Improved virtual orbitals (r4divo.F90:80-93, fockivo.F90:44-270): the Fock matrix of the
// secondary spinors for the state with one electron removed from the HOMO spinors, and its
// eigenvectors per abelian irrep block.
//
// The IVO orbitals written back to DFPCMO are ZHEEV's eigenvectors (diag.F90:66-128), and the
// sign of each is what that algorithm leaves.  So the blocks are diagonalised here by the
// LAPACK 3.x reference algorithm itself, one CTA per block: the Householder reduction ZHETD2
// (upper), the accumulation of Q by ZUNGTR/ZUNG2L, and ZSTEQR's implicit QL/QR iteration with
// Wilkinson shifts, DLAEV2 for 2x2 blocks and the final selection sort.  The Givens generator
// is DLARTG as LAPACK up to 3.9 defines it (the rotation keeps r = sqrt(f^2 + g^2) > 0 unless
// |f| > |g| and f < 0); the reference's IVO outputs carry its signs.  The reductions and the
// rank-2 updates run on all threads of the CTA; the scalar QL/QR recurrence on d and e runs
// in one thread and logs its rotations, which the CTA then applies to the rows of Q in order
// (the rotations never feed back into the recurrence).
#include <algorithm>
#include <vector>

#include "dcg_common.cuh"

namespace dcg {

namespace {

constexpr int kZheevThreads = 256;

struct ZheevJob {
    int n;
    cplx *a;        // n x n, upper triangle read, destroyed
    cplx *z;        // n x n eigenvectors (out)
    double *w;      // n eigenvalues (out), ascending
    cplx *t;        // n
    double *d, *e;  // n, n
    cplx *tau;      // n
    double *rc, *rs;   // rotation log
    int4 *hdr;         // sweep log: first column, length, forward, offset into rc/rs
    int2 *swp;         // selection-sort swaps (n)
    int64_t cap_rot;
    int cap_hdr;
};

__device__ double cta_sum(double v, double *sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); q++) s += sh[q];
        sh[32] = s;
    }
    __syncthreads();
    const double r = sh[32];
    __syncthreads();
    return r;
}

__device__ double dlapy2(double x, double y) {
    const double ax = fabs(x), ay = fabs(y);
    const double w = fmax(ax, ay), z = fmin(ax, ay);
    if (z == 0.0) return w;
    const double q = z / w;
    return w * sqrt(1.0 + q * q);
}

// DLARTG, LAPACK <= 3.9 conventions (without the rescaling of extreme magnitudes).
__device__ void dlartg_v39(double f, double g, double &cs, double &sn, double &r) {
    if (g == 0.0) {
        cs = 1.0;
        sn = 0.0;
        r = f;
        return;
    }
    if (f == 0.0) {
        cs = 0.0;
        sn = 1.0;
        r = g;
        return;
    }
    r = sqrt(f * f + g * g);
    cs = f / r;
    sn = g / r;
    if (fabs(f) > fabs(g) && cs < 0.0) {
        cs = -cs;
        sn = -sn;
        r = -r;
    }
}

// DLAEV2: eigensystem of [[a, b], [b, c]]; (cs1, sn1) is the eigenvector of rt1.
__device__ void dlaev2(double a, double b, double c, double &rt1, double &rt2, double &cs1, double &sn1) {
    const double sm = a + c, df = a - c, adf = fabs(df), tb = b + b, ab = fabs(tb);
    double acmx = c, acmn = a;
    if (fabs(a) > fabs(c)) {
        acmx = a;
        acmn = c;
    }
    double rt;
    if (adf > ab) rt = adf * sqrt(1.0 + (ab / adf) * (ab / adf));
    else if (adf < ab) rt = ab * sqrt(1.0 + (adf / ab) * (adf / ab));
    else rt = ab * sqrt(2.0);
    int sgn1;
    if (sm < 0.0) {
        rt1 = 0.5 * (sm - rt);
        sgn1 = -1;
        rt2 = (acmx / rt1) * acmn - (b / rt1) * b;
    } else if (sm > 0.0) {
        rt1 = 0.5 * (sm + rt);
        sgn1 = 1;
        rt2 = (acmx / rt1) * acmn - (b / rt1) * b;
    } else {
        rt1 = 0.5 * rt;
        rt2 = -0.5 * rt;
        sgn1 = 1;
    }
    int sgn2;
    double cs;
    if (df >= 0.0) {
        cs = df + rt;
        sgn2 = 1;
    } else {
        cs = df - rt;
        sgn2 = -1;
    }
    if (fabs(cs) > ab) {
        const double ct = -tb / cs;
        sn1 = 1.0 / sqrt(1.0 + ct * ct);
        cs1 = ct * sn1;
    } else if (ab == 0.0) {
        cs1 = 1.0;
        sn1 = 0.0;
    } else {
        const double tn = -cs / tb;
        cs1 = 1.0 / sqrt(1.0 + tn * tn);
        sn1 = tn * cs1;
    }
    if (sgn1 == sgn2) {
        const double tn = cs1;
        cs1 = -sn1;
        sn1 = tn;
    }
}

// The scalar part of ZSTEQR (compz 'V') on d (n) and e (n-1); every rotation sequence it
// would apply to Z is appended to the log instead.  Returns 0, 1 (no convergence after 30 n
// sweeps) or 2 (log full).
__device__ int steqr_scalar(int n, double *d, double *e, const ZheevJob &J, int &nh) {
    const double eps = 1.1102230246251565e-16, eps2 = eps * eps, safmin = 2.2250738585072014e-308;
    const int nmaxit = 30 * n;
    int jtot = 0;
    int64_t nr = 0;
    nh = 0;
    auto log_open = [&](int j0, int mm, int fwd) -> int64_t {
        if (nh >= J.cap_hdr || nr + mm > J.cap_rot) return -1;
        J.hdr[nh++] = make_int4(j0, mm, fwd, (int)nr);
        const int64_t at = nr;
        nr += mm - 1;
        return at;
    };
    int l1 = 0;
    while (l1 < n) {
        if (l1 > 0) e[l1 - 1] = 0.0;
        int msplit = n - 1;
        for (int m = l1; m < n - 1; m++) {
            const double tst = fabs(e[m]);
            if (tst == 0.0) {
                msplit = m;
                break;
            }
            if (tst <= sqrt(fabs(d[m])) * sqrt(fabs(d[m + 1])) * eps) {
                e[m] = 0.0;
                msplit = m;
                break;
            }
        }
        int l = l1, lend = msplit;
        const int lsv = l, lendsv = lend;
        l1 = msplit + 1;
        if (lend == l) continue;
        double anorm = 0.0;
        for (int q = l; q <= lend; q++) anorm = fmax(anorm, fabs(d[q]));
        for (int q = l; q < lend; q++) anorm = fmax(anorm, fabs(e[q]));
        if (anorm == 0.0) continue;
        if (fabs(d[lend]) < fabs(d[l])) {
            lend = lsv;
            l = lendsv;
        }
        if (lend > l) {   // QL
            for (;;) {
                int mq = lend;
                for (int m = l; m < lend; m++)
                    if (fabs(e[m]) * fabs(e[m]) <= (eps2 * fabs(d[m])) * fabs(d[m + 1]) + safmin) {
                        mq = m;
                        break;
                    }
                if (mq < lend) e[mq] = 0.0;
                double p = d[l];
                if (mq == l) {
                    d[l] = p;
                    l++;
                    if (l <= lend) continue;
                    break;
                }
                if (mq == l + 1) {
                    double rt1, rt2, c, s;
                    dlaev2(d[l], e[l], d[l + 1], rt1, rt2, c, s);
                    const int64_t at = log_open(l, 2, 0);
                    if (at < 0) return 2;
                    J.rc[at] = c;
                    J.rs[at] = s;
                    d[l] = rt1;
                    d[l + 1] = rt2;
                    e[l] = 0.0;
                    l += 2;
                    if (l <= lend) continue;
                    break;
                }
                if (jtot == nmaxit) break;
                jtot++;
                double g = (d[l + 1] - p) / (2.0 * e[l]);
                double r = dlapy2(g, 1.0);
                g = d[mq] - p + (e[l] / (g + copysign(r, g)));
                double s = 1.0, c = 1.0;
                p = 0.0;
                const int64_t at = log_open(l, mq - l + 1, 0);
                if (at < 0) return 2;
                for (int i = mq - 1; i >= l; i--) {
                    const double f = s * e[i], b = c * e[i];
                    dlartg_v39(g, f, c, s, r);
                    if (i != mq - 1) e[i + 1] = r;
                    g = d[i + 1] - p;
                    r = (d[i] - g) * s + 2.0 * c * b;
                    p = s * r;
                    d[i + 1] = g + p;
                    g = c * r - b;
                    J.rc[at + (i - l)] = c;
                    J.rs[at + (i - l)] = -s;
                }
                d[l] -= p;
                e[l] = g;
            }
        } else {          // QR
            for (;;) {
                int mq = lend;
                for (int m = l; m > lend; m--)
                    if (fabs(e[m - 1]) * fabs(e[m - 1]) <= (eps2 * fabs(d[m])) * fabs(d[m - 1]) + safmin) {
                        mq = m;
                        break;
                    }
                if (mq > lend) e[mq - 1] = 0.0;
                double p = d[l];
                if (mq == l) {
                    d[l] = p;
                    l--;
                    if (l >= lend) continue;
                    break;
                }
                if (mq == l - 1) {
                    double rt1, rt2, c, s;
                    dlaev2(d[l - 1], e[l - 1], d[l], rt1, rt2, c, s);
                    const int64_t at = log_open(l - 1, 2, 1);
                    if (at < 0) return 2;
                    J.rc[at] = c;
                    J.rs[at] = s;
                    d[l - 1] = rt1;
                    d[l] = rt2;
                    e[l - 1] = 0.0;
                    l -= 2;
                    if (l >= lend) continue;
                    break;
                }
                if (jtot == nmaxit) break;
                jtot++;
                double g = (d[l - 1] - p) / (2.0 * e[l - 1]);
                double r = dlapy2(g, 1.0);
                g = d[mq] - p + (e[l - 1] / (g + copysign(r, g)));
                double s = 1.0, c = 1.0;
                p = 0.0;
                const int64_t at = log_open(mq, l - mq + 1, 1);
                if (at < 0) return 2;
                for (int i = mq; i < l; i++) {
                    const double f = s * e[i], b = c * e[i];
                    dlartg_v39(g, f, c, s, r);
                    if (i != mq) e[i - 1] = r;
                    g = d[i] - p;
                    r = (d[i + 1] - g) * s + 2.0 * c * b;
                    p = s * r;
                    d[i] = g + p;
                    g = c * r - b;
                    J.rc[at + (i - mq)] = c;
                    J.rs[at + (i - mq)] = s;
                }
                d[l] -= p;
                e[l - 1] = g;
            }
        }
        if (jtot >= nmaxit) return 1;
    }
    return 0;
}

__global__ void __launch_bounds__(kZheevThreads) zheev_lapack_kernel(const ZheevJob *__restrict__ jobs, int *status) {
    __shared__ double sh[33];
    __shared__ cplx s_tau, s_scal;
    __shared__ int s_skip, s_nh, s_nswp, s_st;
    const ZheevJob J = jobs[blockIdx.x];
    const int n = J.n, tid = threadIdx.x, nt = blockDim.x;
    cplx *a = J.a, *q = J.z, *t = J.t;
    if (n <= 0) return;
    if (n == 1) {
        if (tid == 0) {
            J.w[0] = a[0].x;
            q[0] = mk(1.0, 0.0);
            status[blockIdx.x] = 0;
        }
        return;
    }
    // ---- ZHETD2, uplo 'U'
    if (tid == 0) a[(size_t)(n - 1) * n + (n - 1)].y = 0.0;
    __syncthreads();
    for (int i = n - 2; i >= 0; i--) {
        cplx *col = a + (size_t)(i + 1) * n;
        double xs = 0.0;
        for (int k = tid; k < i; k += nt) xs += cabs2(col[k]);
        xs = cta_sum(xs, sh);
        if (tid == 0) {
            const cplx alpha = col[i];
            const double xnorm = sqrt(xs);
            if (xnorm == 0.0 && alpha.y == 0.0) {
                s_skip = 1;
                s_tau = mk(0.0, 0.0);
                J.e[i] = alpha.x;
            } else {
                const double beta = -copysign(sqrt(alpha.x * alpha.x + alpha.y * alpha.y + xs), alpha.x);
                s_tau = mk((beta - alpha.x) / beta, -alpha.y / beta);
                s_scal = cdiv(mk(1.0, 0.0), mk(alpha.x - beta, alpha.y));
                s_skip = 0;
                J.e[i] = beta;
            }
        }
        __syncthreads();
        const cplx taui = s_tau;
        if (!s_skip) {
            const cplx sc = s_scal;
            for (int k = tid; k < i; k += nt) col[k] = cmul(col[k], sc);
            if (tid == 0) col[i] = mk(1.0, 0.0);
            __syncthreads();
            // t = tau H v over rows 0..i (H from the upper triangle)
            for (int r = tid; r <= i; r += nt) {
                cplx acc = mk(0.0, 0.0);
                for (int c = 0; c <= i; c++) {
                    cplx h;
                    if (r < c) h = a[(size_t)c * n + r];
                    else if (r > c) h = cconj(a[(size_t)r * n + c]);
                    else h = mk(a[(size_t)r * n + r].x, 0.0);
                    acc = cadd(acc, cmul(h, col[c]));
                }
                t[r] = cmul(taui, acc);
            }
            __syncthreads();
            double dre = 0.0, dim = 0.0;
            for (int k = tid; k <= i; k += nt) {
                const cplx u = t[k], v = col[k];
                dre += u.x * v.x + u.y * v.y;
                dim += u.x * v.y - u.y * v.x;
            }
            dre = cta_sum(dre, sh);
            dim = cta_sum(dim, sh);
            const cplx al = cmul(mk(-0.5 * taui.x, -0.5 * taui.y), mk(dre, dim));
            for (int k = tid; k <= i; k += nt) t[k] = cadd(t[k], cmul(al, col[k]));
            __syncthreads();
            const int m1 = i + 1;
            for (int idx = tid; idx < m1 * m1; idx += nt) {
                const int r = idx % m1, c = idx / m1;
                if (r > c) continue;
                cplx &x = a[(size_t)c * n + r];
                x = csub(x, cadd(cmulc(col[r], t[c]), cmulc(t[r], col[c])));
                if (r == c) x.y = 0.0;
            }
            __syncthreads();
        } else if (tid == 0) {
            a[(size_t)i * n + i].y = 0.0;
        }
        __syncthreads();
        if (tid == 0) {
            col[i] = mk(J.e[i], 0.0);
            J.d[i + 1] = a[(size_t)(i + 1) * n + (i + 1)].x;
            J.tau[i] = taui;
        }
        __syncthreads();
    }
    if (tid == 0) J.d[0] = a[0].x;
    // ---- ZUNGTR, uplo 'U': reflector vectors shifted one column left, then ZUNG2L
    for (int idx = tid; idx < n * n; idx += nt) {
        const int r = idx % n, c = idx / n;
        cplx v = mk(0.0, 0.0);
        if (c < n - 1 && r < c) v = a[(size_t)(c + 1) * n + r];
        if (r == n - 1 && c == n - 1) v = mk(1.0, 0.0);
        q[idx] = v;
    }
    __syncthreads();
    const int m = n - 1;
    for (int i = 0; i < m; i++) {
        const cplx ti = J.tau[i];
        if (tid == 0) q[(size_t)i * n + i] = mk(1.0, 0.0);
        __syncthreads();
        if (i > 0) {
            for (int c = tid; c < i; c += nt) {
                cplx acc = mk(0.0, 0.0);
                for (int r = 0; r <= i; r++) acc = cadd(acc, cmulc(q[(size_t)i * n + r], q[(size_t)c * n + r]));
                t[c] = acc;   // (C^H v)_c
            }
            __syncthreads();
            for (int idx = tid; idx < (i + 1) * i; idx += nt) {
                const int r = idx % (i + 1), c = idx / (i + 1);
                q[(size_t)c * n + r] = csub(q[(size_t)c * n + r], cmulc(cmul(ti, q[(size_t)i * n + r]), t[c]));
            }
            __syncthreads();
            for (int r = tid; r < i; r += nt) q[(size_t)i * n + r] = cmul(mk(-ti.x, -ti.y), q[(size_t)i * n + r]);
        }
        __syncthreads();
        if (tid == 0) q[(size_t)i * n + i] = mk(1.0 - ti.x, -ti.y);
        for (int r = i + 1 + tid; r < m; r += nt) q[(size_t)i * n + r] = mk(0.0, 0.0);
        __syncthreads();
    }
    // ---- ZSTEQR: the recurrence in one thread, then its rotations on the rows of Q
    if (tid == 0) {
        int nh = 0;
        s_st = steqr_scalar(n, J.d, J.e, J, nh);
        s_nh = nh;
    }
    __syncthreads();
    const int nh = s_nh;
    for (int r = tid; r < n; r += nt) {
        for (int h = 0; h < nh; h++) {
            const int4 H = J.hdr[h];
            const int j0 = H.x, mm = H.y;
            for (int jj = 0; jj < mm - 1; jj++) {
                const int j = H.z ? jj : (mm - 2 - jj);
                const double ct = J.rc[H.w + j], st = J.rs[H.w + j];
                if (ct == 1.0 && st == 0.0) continue;
                cplx &x0 = q[(size_t)(j0 + j) * n + r];
                cplx &x1 = q[(size_t)(j0 + j + 1) * n + r];
                const cplx tmp = x1;
                x1 = mk(ct * tmp.x - st * x0.x, ct * tmp.y - st * x0.y);
                x0 = mk(st * tmp.x + ct * x0.x, st * tmp.y + ct * x0.y);
            }
        }
    }
    __syncthreads();
    // selection sort of the eigenvalues, swapping eigenvector columns
    if (tid == 0) {
        int ns_ = 0;
        double *d = J.d;
        for (int ii = 1; ii < n; ii++) {
            const int i = ii - 1;
            int k = i;
            double p = d[i];
            for (int j = ii; j < n; j++)
                if (d[j] < p) {
                    k = j;
                    p = d[j];
                }
            if (k != i) {
                d[k] = d[i];
                d[i] = p;
                J.swp[ns_++] = make_int2(i, k);
            }
        }
        s_nswp = ns_;
    }
    __syncthreads();
    for (int r = tid; r < n; r += nt)
        for (int h = 0; h < s_nswp; h++) {
            const int2 S = J.swp[h];
            const cplx x = q[(size_t)S.x * n + r];
            q[(size_t)S.x * n + r] = q[(size_t)S.y * n + r];
            q[(size_t)S.y * n + r] = x;
        }
    for (int k = tid; k < n; k += nt) J.w[k] = J.d[k];
    if (tid == 0) status[blockIdx.x] = s_st;
}

// f (ns x ns, upper triangle) = e_a delta_ab - sum_{k in [k0, k1)} w_k [(ab|kk) - (ak|kb)] / numh
// with w_k = 1/2 for the two highest active spinors when the electron count is odd
// (fockivo.F90:56-85).  F1A = (ab|kl) at a + S (b + S (k + na l)), F2A = (al|kb) at
// a + S (l + na (k + na b)).
__global__ void ivo_fock_kernel(int ns, int na, const cplx *__restrict__ F1A, const cplx *__restrict__ F2A,
                                const double *__restrict__ e_sec, int k0, int k1, int odd, double numh, cplx *f) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)ns * ns) return;
    const int a = (int)(idx % ns), b = (int)(idx / ns);
    if (a > b) {
        f[idx] = mk(0.0, 0.0);
        return;
    }
    const int64_t S = ns;
    cplx v = mk(a == b ? e_sec[a] : 0.0, 0.0);
    for (int k = k0; k < k1; k++) {
        const double w = (odd && k >= na - 2) ? 0.5 : 1.0;
        const cplx g1 = F1A[a + S * (b + S * (k + (int64_t)na * k))];
        const cplx g2 = F2A[a + S * (k + (int64_t)na * (k + (int64_t)na * b))];
        v = csub(v, cscale(g1, w / numh));
        v = cadd(v, cscale(g2, w / numh));
    }
    f[idx] = v;
}

// A_b (n x n, upper) = f[sec_i, sec_j] for the blocks' index lists.
__global__ void ivo_gather_kernel(int ns, const cplx *__restrict__ f, const int *__restrict__ sec, int n,
                                  cplx *A) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)n * n) return;
    const int i = (int)(idx % n), j = (int)(idx / n);
    A[idx] = i <= j ? f[sec[i] + (int64_t)ns * sec[j]] : mk(0.0, 0.0);
}

}  // namespace

void ivo_blocks_eig(Context &c, const cplx *F1A, const cplx *F2A, const double *e_sec_host, int k0, int k1, int odd,
                    double numh, const std::vector<std::vector<int>> &blocks, std::vector<std::vector<double>> &w_out,
                    std::vector<std::vector<cplx>> &v_out) {
    const int ns = c.ns, na = c.na;
    std::vector<double> es(e_sec_host, e_sec_host + ns);
    double *es_d = upload(c, "ivo.es", es);
    cplx *f = wsget<cplx>(c, "ivo.f", (size_t)ns * ns + 1);
    ivo_fock_kernel<<<grid1d((int64_t)ns * ns, 128), 128, 0, c.stream>>>(ns, na, F1A, F2A, es_d, k0, k1, odd, numh, f);
    DCG_LAUNCHED(c);
    const int nb = (int)blocks.size();
    std::vector<ZheevJob> jobs(nb);
    for (int b = 0; b < nb; b++) {
        const int n = (int)blocks[b].size();
        const std::string tg = "#" + std::to_string(b);
        ZheevJob &J = jobs[b];
        J.n = n;
        const size_t nn = (size_t)n * n + 1;
        J.a = wsget<cplx>(c, "ivo.a" + tg, nn);
        J.z = wsget<cplx>(c, "ivo.z" + tg, nn);
        J.t = wsget<cplx>(c, "ivo.t" + tg, (size_t)n + 1);
        J.tau = wsget<cplx>(c, "ivo.tau" + tg, (size_t)n + 1);
        J.w = wsget<double>(c, "ivo.w" + tg, (size_t)n + 1);
        J.d = wsget<double>(c, "ivo.d" + tg, (size_t)n + 1);
        J.e = wsget<double>(c, "ivo.e" + tg, (size_t)n + 1);
        J.cap_rot = 30LL * n * n + n + 16;
        J.cap_hdr = 31 * n + 16;
        J.rc = wsget<double>(c, "ivo.rc" + tg, (size_t)J.cap_rot);
        J.rs = wsget<double>(c, "ivo.rs" + tg, (size_t)J.cap_rot);
        J.hdr = wsget<int4>(c, "ivo.hdr" + tg, (size_t)J.cap_hdr);
        J.swp = wsget<int2>(c, "ivo.swp" + tg, (size_t)n + 1);
        if (n > 0) {
            int *sec = upload(c, "ivo.sec" + tg, blocks[b]);
            ivo_gather_kernel<<<grid1d((int64_t)n * n, 128), 128, 0, c.stream>>>(ns, f, sec, n, J.a);
            DCG_LAUNCHED(c);
        }
    }
    w_out.assign(nb, {});
    v_out.assign(nb, {});
    if (nb == 0) return;
    ZheevJob *jd = upload(c, "ivo.jobs", jobs);
    int *st = wsget<int>(c, "ivo.st", nb);
    DCG_CUDA(cudaMemsetAsync(st, 0, sizeof(int) * nb, c.stream));
    zheev_lapack_kernel<<<nb, kZheevThreads, 0, c.stream>>>(jd, st);
    DCG_LAUNCHED(c);
    std::vector<int> sh = download(c, st, nb);
    for (int b = 0; b < nb; b++) {
        if (sh[b] == 1) throw Error{DCG_E_NUMERIC, "IVO: ZSTEQR did not converge in 30 n sweeps"};
        if (sh[b] == 2) throw Error{DCG_E_NUMERIC, "IVO: ZSTEQR rotation log full"};
        const int n = jobs[b].n;
        w_out[b] = download(c, jobs[b].w, n);
        v_out[b] = download(c, jobs[b].z, (size_t)n * n);
    }
}

}  // namespace dcg
