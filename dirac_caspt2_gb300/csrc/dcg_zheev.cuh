// LAPACK 3.x ZHEEV (jobz 'V', uplo 'U') restated for one CTA: the Householder reduction
// ZHETD2 (upper), the accumulation of Q by ZUNGTR/ZUNG2L, and ZSTEQR's implicit QL/QR
// iteration with Wilkinson shifts, DLAEV2 for 2x2 blocks and the final selection sort, so
// the eigenvector signs are the ones that algorithm leaves.  The Givens generator is DLARTG
// as LAPACK up to 3.9 defines it (the rotation keeps r = sqrt(f^2 + g^2) > 0 unless
// |f| > |g| and f < 0).  The reductions and the rank-2 updates run on all threads of the
// CTA; the scalar QL/QR recurrence on d and e runs in one thread and logs its rotations,
// which the CTA then applies to the rows of Q in order (the rotations never feed back into
// the recurrence).  Used by IVO (dcg_ivo.cu) and by the Davidson step's Rayleigh matrix
// (dcg_davidson.cu).
#pragma once

#include "dcg_common.cuh"

namespace dcg {
namespace zheev_detail {
namespace {   // each translation unit keeps its own copy

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

// The whole ZHEEV (jobz 'V', uplo 'U') of one job in the calling CTA (all its threads call
// it; blockDim.x a multiple of 32, at most 1024).  Returns 0, 1 (no convergence) or 2 (log
// full) in every thread.
__device__ __noinline__ int zheev_cta(const ZheevJob &J) {
    __shared__ double sh[33];
    __shared__ cplx s_tau, s_scal;
    __shared__ int s_skip, s_nh, s_nswp, s_st;
    const int n = J.n, tid = threadIdx.x, nt = blockDim.x;
    cplx *a = J.a, *q = J.z, *t = J.t;
    if (n <= 0) return 0;
    if (n == 1) {
        if (tid == 0) {
            J.w[0] = a[0].x;
            q[0] = mk(1.0, 0.0);
        }
        __syncthreads();
        return 0;
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
    // ---- ZSTEQR: the recurrence in one thread, then its rotations on the rows of Q.  The
    // recurrence is a serial chain through d and e: up to kSteqrSmem entries they sit in
    // shared memory for it (the same arithmetic, a shorter load latency).
    constexpr int kSteqrSmem = 512;
    __shared__ double sd[kSteqrSmem], se[kSteqrSmem];
    const bool in_smem = n <= kSteqrSmem;
    if (in_smem) {
        for (int k = tid; k < n; k += nt) {
            sd[k] = J.d[k];
            se[k] = k + 1 < n ? J.e[k] : 0.0;
        }
        __syncthreads();
    }
    if (tid == 0) {
        int nh = 0;
        s_st = in_smem ? steqr_scalar(n, sd, se, J, nh) : steqr_scalar(n, J.d, J.e, J, nh);
        s_nh = nh;
    }
    __syncthreads();
    if (in_smem)
        for (int k = tid; k < n; k += nt) J.d[k] = sd[k];
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
    __syncthreads();
    return s_st;
}


}  // namespace
}  // namespace zheev_detail
}  // namespace dcg
