// Integral-side kernels: expansion of the MDCINTNEW record stream into dense class
// tensors, the CASCI-state Fock matrix and the core-Fock pieces of the effective
// one-electron terms.
//
// Expansion: every record (ij|kl) stands for 16 integrals, its time-reversal partners on
// each electron and the permutation partners (module_2integrals.F90:395-434); records
// with i == j and k > l are skipped as in the reference readers
// (module_2integrals.F90:393, divide_2_elec_integral_into_subspaces.F90:117).  Each
// partner is stored at its dense position ("=" semantics of the reference arrays).
#include "dcg_common.cuh"
#include "dcg_kernels.cuh"

namespace dcg {

void class_layout(const Context &c, ClassTensor cls[CL_COUNT]) {
    const int n[4] = {0, c.ni, c.na, c.ns};
    auto set = [&](ClassId id, int a, int b, int cc, int d, int diag) {
        ClassTensor &t = cls[id];
        t.sp[0] = a; t.sp[1] = b; t.sp[2] = cc; t.sp[3] = d;
        t.diag = diag;
        if (diag == 0) {
            for (int q = 0; q < 4; q++) t.dim[q] = n[t.sp[q]];
            t.size = (int64_t)t.dim[0] * t.dim[1] * t.dim[2] * t.dim[3];
        } else {
            // stored [a, b, k]: dims (ns, ns, nk)
            t.dim[0] = c.ns; t.dim[1] = c.ns; t.dim[2] = (diag == 1) ? n[cc] : n[b]; t.dim[3] = 1;
            t.size = (int64_t)t.dim[0] * t.dim[1] * t.dim[2];
        }
    };
    set(CL_C1, 3, 2, 2, 2, 0);
    set(CL_C2, 3, 2, 1, 1, 0);
    set(CL_C3, 3, 1, 1, 2, 0);
    set(CL_D1, 3, 1, 2, 2, 0);
    set(CL_D2, 3, 2, 2, 1, 0);
    set(CL_D3, 3, 1, 1, 1, 0);
    set(CL_E, 3, 1, 2, 1, 0);
    set(CL_F, 3, 2, 3, 2, 0);
    set(CL_G, 3, 1, 3, 2, 0);
    set(CL_H, 3, 1, 3, 1, 0);
    set(CL_F1A, 3, 3, 2, 2, 0);
    set(CL_F2A, 3, 2, 2, 3, 0);
    set(CL_F1D, 3, 3, 1, 1, 1);
    set(CL_F2D, 3, 1, 1, 3, 2);
}

struct ScatterParams {
    cplx *ptr[CL_COUNT];
    int dim[CL_COUNT][4];
    int diag[CL_COUNT];
    signed char lut[81];   // pattern code -> class id, -1 none
    int ni, na, ns;
};

__device__ __forceinline__ int space_of(int x, int ni, int na, int ns) {
    return x < ni ? 1 : (x < ni + na ? 2 : (x < ni + na + ns ? 3 : 4));
}

__device__ __forceinline__ void put(const ScatterParams &P, cplx *inttw, int a, int b, int c, int d, cplx v) {
    const int ni = P.ni, na = P.na, ns = P.ns;
    const int sa = space_of(a, ni, na, ns), sb = space_of(b, ni, na, ns), sc = space_of(c, ni, na, ns),
              sd = space_of(d, ni, na, ns);
    if ((sa | sb | sc | sd) & 4) return;   // space 4: beyond nsec
    if (sa <= 2 && sb <= 2 && sc <= 2 && sd <= 2) {
        const int64_t n = ni + na;
        inttw[a + n * (b + n * (c + n * (int64_t)d))] = v;
        return;
    }
    const int code = (sa - 1) * 27 + (sb - 1) * 9 + (sc - 1) * 3 + (sd - 1);
    const int id = P.lut[code];
    if (id < 0) return;
    const int off[4] = {0, 0, ni, ni + na};
    const int la = a - off[sa], lb = b - off[sb], lc = c - off[sc], ld = d - off[sd];
    const int *dm = P.dim[id];
    int64_t pos;
    if (P.diag[id] == 0) {
        pos = la + (int64_t)dm[0] * (lb + (int64_t)dm[1] * (lc + (int64_t)dm[2] * ld));
    } else if (P.diag[id] == 1) {      // (a b | k k)
        if (lc != ld) return;
        pos = la + (int64_t)dm[0] * (lb + (int64_t)dm[1] * lc);
    } else {                           // (a k | k b) stored [a, b, k]
        if (lb != lc) return;
        pos = la + (int64_t)dm[0] * (ld + (int64_t)dm[1] * lb);
    }
    P.ptr[id][pos] = v;
}

__global__ void scatter_kernel(ScatterParams P, const int32_t *__restrict__ ijkl, const cplx *__restrict__ val,
                               int64_t nrec, cplx *inttw) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrec) return;
    const int i = ijkl[4 * r + 0], j = ijkl[4 * r + 1], k = ijkl[4 * r + 2], l = ijkl[4 * r + 3];
    if (i == j && k > l) return;
    const cplx v = val[r], vc = cconj(v);
    // 1-based Kramers partner: odd -> +1, even -> -1
    const int it = (i & 1) ? i + 1 : i - 1, jt = (j & 1) ? j + 1 : j - 1;
    const int kt = (k & 1) ? k + 1 : k - 1, lt = (l & 1) ? l + 1 : l - 1;
    const double sij = ((i + j) & 1) ? -1.0 : 1.0, skl = ((k + l) & 1) ? -1.0 : 1.0;
    const double s2 = sij * skl;
#define P0(a) ((a) - 1)
    put(P, inttw, P0(i), P0(j), P0(k), P0(l), v);
    put(P, inttw, P0(jt), P0(it), P0(k), P0(l), cscale(v, sij));
    put(P, inttw, P0(i), P0(j), P0(lt), P0(kt), cscale(v, skl));
    put(P, inttw, P0(jt), P0(it), P0(lt), P0(kt), cscale(v, s2));
    put(P, inttw, P0(j), P0(i), P0(l), P0(k), vc);
    put(P, inttw, P0(it), P0(jt), P0(l), P0(k), cscale(vc, sij));
    put(P, inttw, P0(j), P0(i), P0(kt), P0(lt), cscale(vc, skl));
    put(P, inttw, P0(it), P0(jt), P0(kt), P0(lt), cscale(vc, s2));
    put(P, inttw, P0(k), P0(l), P0(i), P0(j), v);
    put(P, inttw, P0(lt), P0(kt), P0(i), P0(j), cscale(v, skl));
    put(P, inttw, P0(k), P0(l), P0(jt), P0(it), cscale(v, sij));
    put(P, inttw, P0(lt), P0(kt), P0(jt), P0(it), cscale(v, s2));
    put(P, inttw, P0(l), P0(k), P0(j), P0(i), vc);
    put(P, inttw, P0(kt), P0(lt), P0(j), P0(i), cscale(vc, skl));
    put(P, inttw, P0(l), P0(k), P0(it), P0(jt), cscale(vc, sij));
    put(P, inttw, P0(kt), P0(lt), P0(it), P0(jt), cscale(vc, s2));
#undef P0
}

void launch_scatter(Context &c, const int32_t *ijkl, const cplx *val, int64_t nrec, cplx *inttw,
                    ClassTensor cls[CL_COUNT]) {
    ScatterParams P;
    for (int q = 0; q < 81; q++) P.lut[q] = -1;
    for (int id = 0; id < CL_COUNT; id++) {
        P.ptr[id] = cls[id].p;
        for (int q = 0; q < 4; q++) P.dim[id][q] = cls[id].dim[q];
        P.diag[id] = cls[id].diag;
        const int code = (cls[id].sp[0] - 1) * 27 + (cls[id].sp[1] - 1) * 9 + (cls[id].sp[2] - 1) * 3 + (cls[id].sp[3] - 1);
        P.lut[code] = (signed char)id;
    }
    P.ni = c.ni;
    P.na = c.na;
    P.ns = c.ns;
    if (nrec == 0) return;
    scatter_kernel<<<grid1d(nrec, 256), 256, 0, c.stream>>>(P, ijkl, val, nrec, inttw);
    DCG_LAUNCHED(c);
}

// ------------------------------------------------------------------------- Fock matrix
// f(i,j) for i <= j on the occupied (inactive+active) block and the secondary block,
// hermitian fill of the lower triangle (fockcasci.F90:4-90).  D1act(k,l) = <E_kl>.
__global__ void fock_occ_kernel(int ni, int na, int nmo, const cplx *__restrict__ h, const cplx *__restrict__ g,
                                const cplx *__restrict__ D1, cplx *f) {
    const int nmoc = ni + na;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)nmoc * nmoc) return;
    const int i = (int)(idx % nmoc), j = (int)(idx / nmoc);
    if (i > j) return;
    const int64_t n = nmoc;
#define G(p, q, r, s) g[(p) + n * ((q) + n * ((r) + n * (int64_t)(s)))]
    cplx v = h[i + (int64_t)nmo * j];
    for (int k = 0; k < ni; k++) {
        v = cadd(v, G(i, j, k, k));
        v = csub(v, G(i, k, k, j));
    }
    for (int l = 0; l < na; l++)
        for (int k = 0; k < na; k++) {
            const cplx d = D1[k + (int64_t)na * l];
            v = cadd(v, cmul(d, G(i, j, ni + k, ni + l)));
            v = csub(v, cmul(d, G(i, ni + l, ni + k, j)));
        }
#undef G
    f[i + (int64_t)nmo * j] = v;
    f[j + (int64_t)nmo * i] = cconj(v);
    if (i == j) f[i + (int64_t)nmo * i] = v;
}

__global__ void fock_sec_kernel(int ni, int na, int ns, int nmo, const cplx *__restrict__ h, const cplx *__restrict__ F1A,
                                const cplx *__restrict__ F2A, const cplx *__restrict__ F1D, const cplx *__restrict__ F2D,
                                const cplx *__restrict__ D1, cplx *f) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)ns * ns) return;
    const int a = (int)(idx % ns), b = (int)(idx / ns);
    if (a > b) return;
    const int off = ni + na;
    const int64_t S = ns;
    cplx v = h[(off + a) + (int64_t)nmo * (off + b)];
    for (int k = 0; k < ni; k++) {
        v = cadd(v, F1D[a + S * (b + S * k)]);
        v = csub(v, F2D[a + S * (b + S * k)]);
    }
    for (int l = 0; l < na; l++)
        for (int k = 0; k < na; k++) {
            const cplx d = D1[k + (int64_t)na * l];
            v = cadd(v, cmul(d, F1A[a + S * (b + S * (k + (int64_t)na * l))]));      // (ab|kl)
            v = csub(v, cmul(d, F2A[a + S * (l + (int64_t)na * (k + (int64_t)na * b))]));  // (al|kb)
        }
    f[(off + a) + (int64_t)nmo * (off + b)] = v;
    f[(off + b) + (int64_t)nmo * (off + a)] = cconj(v);
    if (a == b) f[(off + a) + (int64_t)nmo * (off + a)] = v;
}

void launch_fock(Context &c, const cplx *h, const cplx *g, const ClassTensor cls[CL_COUNT], const cplx *D1act,
                 cplx *f) {
    DCG_CUDA(cudaMemsetAsync(f, 0, sizeof(cplx) * (size_t)c.nmo * c.nmo, c.stream));
    const int nmoc = c.ni + c.na;
    if (nmoc > 0) {
        fock_occ_kernel<<<grid1d((int64_t)nmoc * nmoc, 128), 128, 0, c.stream>>>(c.ni, c.na, c.nmo, h, g, D1act, f);
        DCG_LAUNCHED(c);
    }
    if (c.ns > 0) {
        fock_sec_kernel<<<grid1d((int64_t)c.ns * c.ns, 128), 128, 0, c.stream>>>(
            c.ni, c.na, c.ns, c.nmo, h, cls[CL_F1A].p, cls[CL_F2A].p, cls[CL_F1D].p, cls[CL_F2D].p, D1act, f);
        DCG_LAUNCHED(c);
    }
}

// ------------------------------------------------------------------------- core Fock pieces
// Fai(p,i) = h + sum_k [(pi|kk) - (pk|ki)]  (p active, i inactive)      -> effh of A
// Fsi(a,i) = h + sum_k [(ai|kk) - (ak|ki)]  (a secondary, i inactive)   -> effh of D
// Fsa(a,p) = h + sum_k [(ap|kk) - (ak|kp)] - sum_q (aq|qp)              -> effh of C
// (solve_A_subspace.F90 vAmat 546-631, solve_D vDmat, solve_C vCmat).  Summing over the
// untransformed inactive/active spinors equals the reference's sum over the transformed
// ones because both sets span the same space.
__global__ void core_fock_kernel(int ni, int na, int ns, int nmo, const cplx *__restrict__ h, const cplx *__restrict__ g,
                                 const cplx *__restrict__ C1, const cplx *__restrict__ C2, const cplx *__restrict__ C3,
                                 const cplx *__restrict__ D3, cplx *Fai, cplx *Fsi, cplx *Fsa) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nai = (int64_t)na * ni, nsi = (int64_t)ns * ni, nsa = (int64_t)ns * na;
    const int64_t n = ni + na;
#define G(p, q, r, s) g[(p) + n * ((q) + n * ((r) + n * (int64_t)(s)))]
    if (idx < nai) {
        const int p = (int)(idx % na), i = (int)(idx / na);
        cplx v = h[(ni + p) + (int64_t)nmo * i];
        for (int k = 0; k < ni; k++) {
            v = cadd(v, G(ni + p, i, k, k));
            v = csub(v, G(ni + p, k, k, i));
        }
        Fai[idx] = v;
        return;
    }
    int64_t r = idx - nai;
    const int64_t S = ns, A = na, I = ni;
    if (r < nsi) {
        const int a = (int)(r % ns), i = (int)(r / ns);
        cplx v = h[(n + a) + (int64_t)nmo * i];
        for (int k = 0; k < ni; k++) {
            v = cadd(v, D3[a + S * (i + I * (k + I * k))]);
            v = csub(v, D3[a + S * (k + I * (k + I * i))]);
        }
        Fsi[r] = v;
        return;
    }
    r -= nsi;
    if (r < nsa) {
        const int a = (int)(r % ns), p = (int)(r / ns);
        cplx v = h[(n + a) + (int64_t)nmo * (ni + p)];
        for (int k = 0; k < ni; k++) {
            v = cadd(v, C2[a + S * (p + A * (k + I * k))]);      // (ap|kk)
            v = csub(v, C3[a + S * (k + I * (k + I * p))]);      // (ak|kp)
        }
        for (int q = 0; q < na; q++) v = csub(v, C1[a + S * (q + A * (q + A * p))]);   // (aq|qp)
        Fsa[r] = v;
    }
#undef G
}

void launch_core_fock(Context &c, const cplx *h, const cplx *g, const ClassTensor cls[CL_COUNT], cplx *Fai, cplx *Fsi,
                      cplx *Fsa) {
    const int64_t tot = (int64_t)c.na * c.ni + (int64_t)c.ns * c.ni + (int64_t)c.ns * c.na;
    if (tot == 0) return;
    core_fock_kernel<<<grid1d(tot, 128), 128, 0, c.stream>>>(c.ni, c.na, c.ns, c.nmo, h, g, cls[CL_C1].p, cls[CL_C2].p,
                                                             cls[CL_C3].p, cls[CL_D3].p, Fai, Fsi, Fsa);
    DCG_LAUNCHED(c);
}

// ------------------------------------------------------------------------- small helpers
__global__ void subblock_kernel(const cplx *__restrict__ g, int64_t n, int o0, int o1, int o2, int o3, int d0, int d1,
                                int d2, int d3, cplx *out) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t tot = (int64_t)d0 * d1 * d2 * d3;
    if (idx >= tot) return;
    int64_t r = idx;
    const int i = (int)(r % d0); r /= d0;
    const int j = (int)(r % d1); r /= d1;
    const int k = (int)(r % d2); r /= d2;
    const int l = (int)r;
    out[idx] = g[(o0 + i) + n * ((o1 + j) + n * ((o2 + k) + n * (int64_t)(o3 + l)))];
}

void launch_subblock(Context &c, const cplx *g, int nmoc, const int off[4], const int dim[4], cplx *out) {
    const int64_t tot = (int64_t)dim[0] * dim[1] * dim[2] * dim[3];
    if (tot == 0) return;
    subblock_kernel<<<grid1d(tot, 256), 256, 0, c.stream>>>(g, nmoc, off[0], off[1], off[2], off[3], dim[0], dim[1],
                                                            dim[2], dim[3], out);
    DCG_LAUNCHED(c);
}

__global__ void zero_small_kernel(cplx *x, int64_t n, double thr) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    if (sqrt(cabs2(x[i])) < thr) x[i] = mk(0.0, 0.0);
}

void launch_zero_small(Context &c, cplx *x, int64_t n, double thr) {
    if (n == 0) return;
    zero_small_kernel<<<grid1d(n, 256), 256, 0, c.stream>>>(x, n, thr);
    DCG_LAUNCHED(c);
}

__global__ void gather2_kernel(const cplx *__restrict__ A, int64_t lda, const int *__restrict__ idx, int n, cplx *out) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)n * n) return;
    const int i = (int)(q % n), j = (int)(q / n);
    out[q] = A[idx[i] + lda * idx[j]];
}

void launch_gather2(Context &c, const cplx *A, int64_t lda, const int *idx, int n, cplx *out) {
    if (n == 0) return;
    gather2_kernel<<<grid1d((int64_t)n * n, 256), 256, 0, c.stream>>>(A, lda, idx, n, out);
    DCG_LAUNCHED(c);
}

__global__ void scatter2_kernel(const cplx *__restrict__ X, int n, const int *__restrict__ idx, cplx *A, int64_t lda) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)n * n) return;
    const int i = (int)(q % n), j = (int)(q / n);
    A[idx[i] + lda * idx[j]] = X[q];
}

void launch_scatter2(Context &c, const cplx *X, int n, const int *idx, cplx *A, int64_t lda) {
    if (n == 0) return;
    scatter2_kernel<<<grid1d((int64_t)n * n, 256), 256, 0, c.stream>>>(X, n, idx, A, lda);
    DCG_LAUNCHED(c);
}

// Z(:, j) *= w[woff + j]^(-1/2)   (ulambda_s_half.F90:14-75)
__global__ void scale_cols_kernel(cplx *Z, int64_t ldz, int n, int m, const double *w, int woff) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)n * m) return;
    const int i = (int)(q % n), j = (int)(q / n);
    const double s = pow(w[woff + j], -0.5);
    Z[i + ldz * j] = cscale(Z[i + ldz * j], s);
}

void launch_scale_cols(Context &c, cplx *Z, int64_t ldz, int n, int m, const double *w, int woff) {
    if ((int64_t)n * m == 0) return;
    scale_cols_kernel<<<grid1d((int64_t)n * m, 256), 256, 0, c.stream>>>(Z, ldz, n, m, w, woff);
    DCG_LAUNCHED(c);
}

}  // namespace dcg
