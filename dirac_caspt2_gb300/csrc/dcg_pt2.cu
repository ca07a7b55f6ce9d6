// Subspace kernels of CASPT2: S and B matrix assembly from the dense density tensors,
// the V (right-hand side) builds, the E2 reduction and the streaming H subspace.
//
// Density tensors (all from GEMMs over excited CI vectors, see dcg_api.cu):
//   D1(a,b)         = <0|E_ab|0>                                 g1[a + na b]
//   D2(a,b,c,d)     = <0|E_ab E_cd|0>                            g2[(b + na a) + na^2 (c + na d)]
//   D3(a,b,c,d,e,f) = <0|E_ab E_cd E_ef|0>                       g3[(b + na a) + na^2 ((c + na d) + na^2 (e + na f))]
//   T1, T2, T3      = same with F = sum_w eps_w E_ww rightmost, i.e. the reference's
//                     sum_w eps(w) dim(n+1)_density(..., w, w)   t1, t2, t3
#include "dcg_common.cuh"
#include "dcg_kernels.cuh"

namespace dcg {

struct RD {
    const cplx *g1, *g2, *g3, *t1, *t2, *t3;
    int na;
    __device__ __forceinline__ int64_t i2(int a, int b, int c, int d) const {
        const int64_t n2 = (int64_t)na * na;
        return (b + (int64_t)na * a) + n2 * (c + (int64_t)na * d);
    }
    __device__ __forceinline__ int64_t i3(int a, int b, int c, int d, int e, int f) const {
        const int64_t n2 = (int64_t)na * na;
        return (b + (int64_t)na * a) + n2 * ((c + (int64_t)na * d) + n2 * (e + (int64_t)na * f));
    }
    __device__ __forceinline__ cplx D1(int a, int b) const { return g1[a + (int64_t)na * b]; }
    __device__ __forceinline__ cplx T1(int a, int b) const { return t1[a + (int64_t)na * b]; }
    __device__ __forceinline__ cplx D2(int a, int b, int c, int d) const { return g2[i2(a, b, c, d)]; }
    __device__ __forceinline__ cplx T2(int a, int b, int c, int d) const { return t2[i2(a, b, c, d)]; }
    __device__ __forceinline__ cplx D3(int a, int b, int c, int d, int e, int f) const { return g3[i3(a, b, c, d, e, f)]; }
    __device__ __forceinline__ cplx T3(int a, int b, int c, int d, int e, int f) const { return t3[i3(a, b, c, d, e, f)]; }
};

static RD rd_of(const RDMView &r) {
    RD x;
    x.g1 = r.g1; x.g2 = r.g2; x.g3 = r.g3; x.t1 = r.t1; x.t2 = r.t2; x.t3 = r.t3; x.na = r.na;
    return x;
}

__device__ __forceinline__ cplx neg(cplx a) { return mk(-a.x, -a.y); }

// ------------------------------------------------------------------------- S and B
// Upper triangle computed from the reference formula, lower triangle = conj (the
// reference fills sc(j,i) = conj(sc(i,j)); ZHEEV(uplo='U') reads the upper triangle).
template <char SUB>
__global__ void sb_kernel(RD r, const int *__restrict__ ind, int dimn, const double *__restrict__ eps, double e0, cplx *S,
                          cplx *B) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)dimn * dimn) return;
    const int i = (int)(q % dimn), j = (int)(q / dimn);
    if (i > j) return;
    cplx s = mk(0.0, 0.0), b = mk(0.0, 0.0);
    if (SUB == 'A') {   // solve_A_subspace.F90 sAmat 286-338, bAmat 343-424
        const int x = ind[3 * i], y = ind[3 * i + 1], z = ind[3 * i + 2];
        const int t = ind[3 * j], u = ind[3 * j + 1], v = ind[3 * j + 2];
        s = neg(r.D3(z, y, t, x, u, v));
        b = neg(r.T3(z, y, t, x, u, v));
        if (t == x) {
            s = cadd(s, r.D2(z, y, u, v));
            b = cadd(b, r.T2(z, y, u, v));
        }
        b = cadd(b, cscale(s, eps[u] + eps[t] - eps[v]));
    } else if (SUB == 'B') {   // solve_B_subspace.F90 sBmat 294-362, bBmat 367-462
        const int x = ind[2 * i], y = ind[2 * i + 1];
        const int t = ind[2 * j], u = ind[2 * j + 1];
        s = r.D2(t, x, u, y);
        b = r.T2(t, x, u, y);
        if (t == x) { s = csub(s, r.D1(u, y)); b = csub(b, r.T1(u, y)); }
        if (u == y) { s = csub(s, r.D1(t, x)); b = csub(b, r.T1(t, x)); }
        if (t == y) { s = csub(s, r.D1(u, x)); b = csub(b, r.T1(u, x)); }
        if (t == x && u == y) { s = cadd(s, mk(1.0, 0.0)); b = cadd(b, mk(e0, 0.0)); }
        b = cadd(b, cscale(s, eps[t] + eps[u]));
    } else if (SUB == 'C') {   // solve_C_subspace.F90 sCmat 284-338, bCmat 343-422
        const int x = ind[3 * i], y = ind[3 * i + 1], z = ind[3 * i + 2];
        const int t = ind[3 * j], u = ind[3 * j + 1], v = ind[3 * j + 2];
        s = r.D3(z, y, x, t, u, v);
        b = cadd(r.T3(z, y, x, t, u, v), cscale(s, eps[u] - eps[v] - eps[t]));
    } else if (SUB == 'D') {   // solve_D_subspace.F90 sDmat 305-350, bDmat 355-421
        const int x = ind[2 * i], y = ind[2 * i + 1];
        const int t = ind[2 * j], u = ind[2 * j + 1];
        s = r.D2(y, x, t, u);
        b = cadd(r.T2(y, x, t, u), cscale(s, eps[t] - eps[u]));
    } else if (SUB == 'E') {   // solve_E_subspace.F90 sEmat 281-331, bEmat 336-403
        const int u = ind[i], t = ind[j];
        s = neg(r.D1(t, u));
        b = neg(r.T1(t, u));
        if (u == t) { s = cadd(s, mk(1.0, 0.0)); b = cadd(b, mk(e0, 0.0)); }
        b = cadd(b, cscale(s, eps[t]));
    } else if (SUB == 'F') {   // solve_F_subspace.F90 sFmat 303-356, bFmat 361-437
        const int v = ind[2 * i], x = ind[2 * i + 1];
        const int t = ind[2 * j], u = ind[2 * j + 1];
        s = r.D2(v, t, x, u);
        b = r.T2(v, t, x, u);
        if (x == t) { s = csub(s, r.D1(v, u)); b = csub(b, r.T1(v, u)); }
        b = cadd(b, cscale(s, -eps[u] - eps[t]));
    } else if (SUB == 'G') {   // solve_G_subspace.F90 sGmat 295-337, bGmat 342-405
        const int t = ind[i], u = ind[j];
        s = r.D1(t, u);
        b = csub(r.T1(t, u), cscale(s, eps[t]));
    }
    S[i + (int64_t)dimn * j] = s;
    B[i + (int64_t)dimn * j] = b;
    if (i != j) {
        S[j + (int64_t)dimn * i] = cconj(s);
        B[j + (int64_t)dimn * i] = cconj(b);
    } else {
        S[i + (int64_t)dimn * i].y = 0.0;
        B[i + (int64_t)dimn * i].y = 0.0;
    }
}

void launch_SB(Context &c, char sub, const RDMView &rv, const int *ind, int dimn, const double *eps_act, double e0,
               cplx *S, cplx *B) {
    RD r = rd_of(rv);
    const int64_t n2 = (int64_t)dimn * dimn;
    const unsigned g = grid1d(n2, 256);
    switch (sub) {
        case 'A': sb_kernel<'A'><<<g, 256, 0, c.stream>>>(r, ind, dimn, eps_act, e0, S, B); break;
        case 'B': sb_kernel<'B'><<<g, 256, 0, c.stream>>>(r, ind, dimn, eps_act, e0, S, B); break;
        case 'C': sb_kernel<'C'><<<g, 256, 0, c.stream>>>(r, ind, dimn, eps_act, e0, S, B); break;
        case 'D': sb_kernel<'D'><<<g, 256, 0, c.stream>>>(r, ind, dimn, eps_act, e0, S, B); break;
        case 'E': sb_kernel<'E'><<<g, 256, 0, c.stream>>>(r, ind, dimn, eps_act, e0, S, B); break;
        case 'F': sb_kernel<'F'><<<g, 256, 0, c.stream>>>(r, ind, dimn, eps_act, e0, S, B); break;
        case 'G': sb_kernel<'G'><<<g, 256, 0, c.stream>>>(r, ind, dimn, eps_act, e0, S, B); break;
        default: throw Error{DCG_E_ARG, "launch_SB: bad subspace"};
    }
    DCG_LAUNCHED(c);
}

// ------------------------------------------------------------------------- V selection + E2
__global__ void gather_v_kernel(const cplx *__restrict__ V, const int64_t *__restrict__ oo, int nouter,
                                const int64_t *__restrict__ io, int dimn, cplx *Vsel) {
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)dimn * nouter) return;
    const int d = (int)(q % dimn);
    const int64_t o = q / dimn;
    Vsel[q] = V[oo[o] + io[d]];
}

void launch_gather_v(Context &c, const cplx *V, const int64_t *outer_off, int nouter, const int64_t *inner_off,
                     int dimn, cplx *Vsel) {
    const int64_t n = (int64_t)dimn * nouter;
    if (n == 0) return;
    gather_v_kernel<<<grid1d(n, 256), 256, 0, c.stream>>>(V, outer_off, nouter, inner_off, dimn, Vsel);
    DCG_LAUNCHED(c);
}

// e2o[o] = -sum_j |VC(j,o)|^2/(alpha_o + wb_j), sc2o[o] = sum_j |VC(j,o)|^2/(alpha_o + wb_j)^2
// (solve_A_subspace.F90:236-261, same loop in B..G)
__global__ void e2_kernel(const cplx *__restrict__ VC, int dimm, int nouter, const double *__restrict__ alpha,
                          const double *__restrict__ wb, double *e2o, double *sc2o) {
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= nouter) return;
    const double al = alpha[o];
    double e = 0.0, s = 0.0;
    for (int j = 0; j < dimm; j++) {
        const double a2 = cabs2(VC[j + (int64_t)dimm * o]);
        const double den = al + wb[j];
        e -= a2 / den;
        s += a2 / (den * den);
    }
    e2o[o] = e;
    sc2o[o] = s;
}

void launch_e2(Context &c, const cplx *VC, int dimm, int nouter, const double *alpha, const double *wb, double *e2o,
               double *sc2o) {
    if (nouter == 0) return;
    e2_kernel<<<grid1d(nouter, 128), 128, 0, c.stream>>>(VC, dimm, nouter, alpha, wb, e2o, sc2o);
    DCG_LAUNCHED(c);
}

// ------------------------------------------------------------------------- V builds
// B: V[pr + np (x + na y)] for inactive pairs i > j (pr), from R(t,u) = (t i|u j)
// (solve_B_subspace.F90 vBmat 467-591).  Bc: (na, ni, na, ni) transformed.
__global__ void v_B_kernel(RD r, const cplx *__restrict__ Bc, int ni, cplx *V) {
    const int na = r.na;
    const int np = ni * (ni - 1) / 2;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= (int64_t)np * na * na) return;
    const int pr = (int)(q % np);
    const int x = (int)((q / np) % na), y = (int)(q / ((int64_t)np * na));
    int i = 1, cnt = pr;
    while (cnt >= i) { cnt -= i; i++; }
    const int j = cnt;   // pairs ordered (1,0),(2,0),(2,1),(3,0)...
    const int64_t A = na, I = ni;
#define R(t, u) Bc[(t) + A * ((int64_t)i + I * ((u) + A * (int64_t)j))]
    cplx v = csub(R(x, y), R(y, x));
    for (int u = 0; u < na; u++) {
        v = cadd(v, cmul(R(y, u), r.D1(u, x)));
        v = csub(v, cmul(R(x, u), r.D1(u, y)));
        v = csub(v, cmul(R(u, y), r.D1(u, x)));
    }
    for (int u = 0; u < na; u++)
        for (int t = 0; t < na; t++) v = cadd(v, cmul(R(t, u), r.D2(t, x, u, y)));
#undef R
    V[q] = v;
}

void launch_v_B(Context &c, const RDMView &rv, const cplx *Bc, int ni, cplx *V) {
    const int64_t n = (int64_t)(ni * (ni - 1) / 2) * rv.na * rv.na;
    if (n == 0) return;
    v_B_kernel<<<grid1d(n, 128), 128, 0, c.stream>>>(rd_of(rv), Bc, ni, V);
    DCG_LAUNCHED(c);
}

// D: V[(a + ns i) + ns ni (t + na u)] = sum_kl (ai|kl) D2(u,t,k,l) - sum_jk (aj|ki) D2(u,t,k,j)
//    + effh(a,i) D1(u,t)   (solve_D_subspace.F90 vDmat 426-609)
// as one FP64 product: with X[(a,i),(k,l)] = (ai|kl) - (al|ki) (the second sum renamed j -> l)
// and D2 viewed as the na^2 x na^2 matrix G2[(t,u),(k,l)], V = X G2^T + effh (x) D1.  Forming X
// first halves the FP64 operations of the contraction (one complex product per (k,l) instead
// of two), and the product runs on the tuned GEMM.
__global__ void v_D_x_kernel(const cplx *__restrict__ D1c, const cplx *__restrict__ D2c, int ni, int ns, int na,
                             cplx *X) {
    const int64_t nsi = (int64_t)ns * ni;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nsi * na * na) return;
    const int a = (int)(q % ns), i = (int)((q / ns) % ni);
    const int k = (int)((q / nsi) % na), l = (int)(q / (nsi * na));
    const int64_t S = ns, A = na;
    X[q] = csub(D1c[q], D2c[a + S * (l + A * (k + A * (int64_t)i))]);
}

__global__ void v_D_effh_kernel(RD r, const cplx *__restrict__ effh, int ni, int ns, cplx *V) {
    const int na = r.na;
    const int64_t nsi = (int64_t)ns * ni;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nsi * na * na) return;
    const int64_t ai = q % nsi;
    const int t = (int)((q / nsi) % na), u = (int)(q / (nsi * na));
    V[q] = cadd(V[q], cmul(effh[ai], r.D1(u, t)));
}

void launch_v_D(Context &c, const RDMView &rv, const cplx *D1c, const cplx *D2c, const cplx *effh, int ni, int ns,
                cplx *V) {
    const int na = rv.na;
    const int64_t nsi = (int64_t)ns * ni, n = nsi * na * na;
    if (n == 0) return;
    cplx *X = wsget<cplx>(c, "v.Dx", (size_t)n);
    v_D_x_kernel<<<grid1d(n, 256), 256, 0, c.stream>>>(D1c, D2c, ni, ns, na, X);
    DCG_LAUNCHED(c);
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
    zgemm(c, OP_N, OP_T, (int)nsi, na * na, na * na, one, X, nsi, 0, rv.g2, (int64_t)na * na, 0, zero, V, nsi, 0, 1);
    v_D_effh_kernel<<<grid1d(n, 256), 256, 0, c.stream>>>(rd_of(rv), effh, ni, ns, V);
    DCG_LAUNCHED(c);
}

// E: V[(a + ns pr) + ns np t] with pr the inactive pair i > j:
//    -(ai|tj) + (aj|ti) + sum_p D1(t,p) [(ai|pj) - (aj|pi)]   (solve_E_subspace.F90 vEmat 408-476)
__global__ void v_E_kernel(RD r, const cplx *__restrict__ Ec, int ni, int ns, cplx *V) {
    const int na = r.na;
    const int np = ni * (ni - 1) / 2;
    const int64_t nq = (int64_t)ns * np;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq * na) return;
    const int a = (int)(q % ns);
    const int pr = (int)((q / ns) % np);
    const int t = (int)(q / nq);
    int i = 1, cnt = pr;
    while (cnt >= i) { cnt -= i; i++; }
    const int j = cnt;
    const int64_t S = ns, I = ni, A = na;
#define EC(a_, i_, p_, j_) Ec[(a_) + S * ((i_) + I * ((p_) + A * (int64_t)(j_)))]
    cplx v = csub(EC(a, j, t, i), EC(a, i, t, j));
    for (int p = 0; p < na; p++) v = cadd(v, cmul(r.D1(t, p), csub(EC(a, i, p, j), EC(a, j, p, i))));
#undef EC
    V[q] = v;
}

void launch_v_E(Context &c, const RDMView &rv, const cplx *Ec, int ni, int ns, cplx *V) {
    const int64_t n = (int64_t)ns * (ni * (ni - 1) / 2) * rv.na;
    if (n == 0) return;
    v_E_kernel<<<grid1d(n, 128), 128, 0, c.stream>>>(rd_of(rv), Ec, ni, ns, V);
    DCG_LAUNCHED(c);
}

// G: V[(pab + nab i) + nab ni t] with pab the secondary pair a > b:
//    sum_p D1(t,p) [(ai|bp) - (bi|ap)]   (solve_G_subspace.F90 vGmat 410-469)
__global__ void v_G_kernel(RD r, const cplx *__restrict__ Gc, int ni, int ns, cplx *V) {
    const int na = r.na;
    const int64_t nab = (int64_t)ns * (ns - 1) / 2;
    const int64_t nq = nab * ni;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= nq * na) return;
    const int64_t pab = q % nab;
    const int i = (int)((q / nab) % ni);
    const int t = (int)(q / nq);
    // pab -> (a, b), a > b, ordered (1,0),(2,0),(2,1),...
    int a = (int)floor((1.0 + sqrt(1.0 + 8.0 * (double)pab)) * 0.5);
    while ((int64_t)a * (a - 1) / 2 > pab) a--;
    while ((int64_t)(a + 1) * a / 2 <= pab) a++;
    const int b = (int)(pab - (int64_t)a * (a - 1) / 2);
    const int64_t S = ns, I = ni;
#define GC(a_, i_, b_, p_) Gc[(a_) + S * ((i_) + I * ((b_) + S * (int64_t)(p_)))]
    cplx v = mk(0.0, 0.0);
    for (int p = 0; p < na; p++) v = cadd(v, cmul(r.D1(t, p), csub(GC(a, i, b, p), GC(b, i, a, p))));
#undef GC
    V[q] = v;
}

void launch_v_G(Context &c, const RDMView &rv, const cplx *Gc, int ni, int ns, cplx *V) {
    const int64_t n = (int64_t)ns * (ns - 1) / 2 * ni * rv.na;
    if (n == 0) return;
    v_G_kernel<<<grid1d(n, 128), 128, 0, c.stream>>>(rd_of(rv), Gc, ni, ns, V);
    DCG_LAUNCHED(c);
}

// A: P3[(p + na(q + na r)) + na^3 (t + na(u + na v))] = D3(v,u,p,t,q,r)
__global__ void perm_A_kernel(RD r, cplx *P3) {
    const int na = r.na;
    const int64_t n3 = (int64_t)na * na * na;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n3 * n3) return;
    int64_t x = q;
    const int p = (int)(x % na); x /= na;
    const int qq = (int)(x % na); x /= na;
    const int rr = (int)(x % na); x /= na;
    const int t = (int)(x % na); x /= na;
    const int u = (int)(x % na); x /= na;
    const int v = (int)x;
    P3[q] = r.D3(v, u, p, t, qq, rr);
}

// C: P3[(j + na(k + na l)) + na^3 (t + na(u + na v))] = D3(v,u,t,j,k,l)
//    P2[p + na (t + na(u + na v))] = D2(v,u,t,p)
__global__ void perm_C_kernel(RD r, cplx *P3, cplx *P2) {
    const int na = r.na;
    const int64_t n3 = (int64_t)na * na * na;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n3 * n3) return;
    int64_t x = q;
    const int j = (int)(x % na); x /= na;
    const int k = (int)(x % na); x /= na;
    const int l = (int)(x % na); x /= na;
    const int t = (int)(x % na); x /= na;
    const int u = (int)(x % na); x /= na;
    const int v = (int)x;
    P3[q] = r.D3(v, u, t, j, k, l);
    if (q < (int64_t)na * n3) {
        int64_t y = q;
        const int p = (int)(y % na); y /= na;
        const int t2 = (int)(y % na); y /= na;
        const int u2 = (int)(y % na); y /= na;
        const int v2 = (int)y;
        P2[q] = r.D2(v2, u2, t2, p);
    }
}

// F: P2[(p + na q) + na^2 (x + na y)] = D2(x,p,y,q) - delta(p,y) D1(x,q)
__global__ void perm_F_kernel(RD r, cplx *P2) {
    const int na = r.na;
    const int64_t n2 = (int64_t)na * na;
    const int64_t q0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q0 >= n2 * n2) return;
    int64_t x0 = q0;
    const int p = (int)(x0 % na); x0 /= na;
    const int q = (int)(x0 % na); x0 /= na;
    const int x = (int)(x0 % na); x0 /= na;
    const int y = (int)x0;
    cplx v = r.D2(x, p, y, q);
    if (p == y) v = csub(v, r.D1(x, q));
    P2[q0] = v;
}

void launch_perm_A(Context &c, const RDMView &rv, cplx *P3, cplx *) {
    const int64_t n3 = (int64_t)rv.na * rv.na * rv.na;
    perm_A_kernel<<<grid1d(n3 * n3, 256), 256, 0, c.stream>>>(rd_of(rv), P3);
    DCG_LAUNCHED(c);
}

void launch_perm_C2(Context &c, const RDMView &rv, cplx *P3, cplx *P2) {
    const int64_t n3 = (int64_t)rv.na * rv.na * rv.na;
    perm_C_kernel<<<grid1d(n3 * n3, 256), 256, 0, c.stream>>>(rd_of(rv), P3, P2);
    DCG_LAUNCHED(c);
}

void launch_perm_F(Context &c, const RDMView &rv, cplx *P2, cplx *) {
    const int64_t n2 = (int64_t)rv.na * rv.na;
    perm_F_kernel<<<grid1d(n2 * n2, 256), 256, 0, c.stream>>>(rd_of(rv), P2);
    DCG_LAUNCHED(c);
}

// A remainder: V(i,t,u,v) += sum_pq (ti|pq) D2(v,u,p,q) + effh(t,i) D1(v,u) - sum_p effh(p,i) D2(v,u,p,t)
// A1: (na, ni, na, na) transformed; effh: (na, ni).  V layout i + ni (t + na (u + na v)).
__global__ void v_A_rest_kernel(RD r, const cplx *__restrict__ A1, const cplx *__restrict__ effh, int ni, cplx *V) {
    const int na = r.na;
    const int64_t tot = (int64_t)ni * na * na * na;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= tot) return;
    int64_t x = q;
    const int i = (int)(x % ni); x /= ni;
    const int t = (int)(x % na); x /= na;
    const int u = (int)(x % na); x /= na;
    const int v = (int)x;
    const int64_t A = na, I = ni;
    cplx acc = cmul(effh[t + A * i], r.D1(v, u));
    for (int qq = 0; qq < na; qq++)
        for (int p = 0; p < na; p++)
            acc = cadd(acc, cmul(A1[t + A * (i + I * (p + A * (int64_t)qq))], r.D2(v, u, p, qq)));
    for (int p = 0; p < na; p++) acc = csub(acc, cmul(effh[p + A * i], r.D2(v, u, p, t)));
    V[q] = cadd(V[q], acc);
}

void launch_v_A_rest(Context &c, const RDMView &rv, const cplx *A1, const cplx *effh, int ni, cplx *V) {
    const int64_t tot = (int64_t)ni * rv.na * rv.na * rv.na;
    if (tot == 0) return;
    v_A_rest_kernel<<<grid1d(tot, 128), 128, 0, c.stream>>>(rd_of(rv), A1, effh, ni, V);
    DCG_LAUNCHED(c);
}

// A1p[i + ni (p + na (q + na r))] = A1[p + na (i + ni (q + na r))]
__global__ void permute_A1_kernel(const cplx *__restrict__ A1, int na, int ni, cplx *A1p) {
    const int64_t tot = (int64_t)ni * na * na * na;
    const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= tot) return;
    int64_t x = q;
    const int i = (int)(x % ni); x /= ni;
    const int p = (int)(x % na); x /= na;
    const int64_t rest = x;   // q + na r
    A1p[q] = A1[p + (int64_t)na * (i + (int64_t)ni * rest)];
}

void launch_permute_A1(Context &c, const cplx *A1, int na, int ni, cplx *A1p) {
    const int64_t tot = (int64_t)ni * na * na * na;
    if (tot == 0) return;
    permute_A1_kernel<<<grid1d(tot, 256), 256, 0, c.stream>>>(A1, na, ni, A1p);
    DCG_LAUNCHED(c);
}

// Fp[(a + ns b) + ns^2 (p + na q)] = F[a + ns (p + na (b + ns q))]
__global__ void F_pack_kernel(const cplx *__restrict__ Fc, int ns, int na, cplx *Fp) {
    const int64_t S = ns, A = na;
    const int64_t tot = S * S * A * A;
    const int64_t q0 = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (q0 >= tot) return;
    int64_t x = q0;
    const int a = (int)(x % S); x /= S;
    const int b = (int)(x % S); x /= S;
    const int p = (int)(x % A); x /= A;
    const int q = (int)x;
    Fp[q0] = Fc[a + S * (p + A * (b + S * q))];
}

void launch_F_pack(Context &c, const cplx *Fc, int ns, int na, cplx *Fp) {
    const int64_t tot = (int64_t)ns * ns * na * na;
    if (tot == 0) return;
    F_pack_kernel<<<grid1d(tot, 256), 256, 0, c.stream>>>(Fc, ns, na, Fp);
    DCG_LAUNCHED(c);
}

// ------------------------------------------------------------------------- H subspace
// e2h = -sum |V|^2/e, sumc2 = sum |V/e|^2 over a > b, i > j with
// V = (ai|bj) - (aj|bi), e = eps_a + eps_b - eps_i - eps_j + eshift and the symmetry
// condition MULTB_S(MULTB_D(irp a, irp i), MULTB_D(irp b, irp j)) == 1
// (solve_H_subspace.F90:119-175).  Hc: (ns, ni, ns, ni), (a i|b j) at a + ns (i + ni (b + ns j)).
//
// One block per (b, i), i >= 1: its threads run over the (j < i, a > b) pairs with a fastest, so
// both operands, (a i|b j) and (a j|b i), are contiguous runs over a and every element of the
// a > b half of the class is read exactly once (streaming loads); the a < b half is never read.
// The FP64 pipe, not HBM, bounds this kernel on GB300 (about two FP64 operations per clock per
// SM): per element two subtractions and |V|^2, the denominator, a reciprocal and the two
// accumulations.  The reciprocal is the FP32 one widened and refined by one Newton-Raphson step
// for 1/e, r = r0 + r0 (1 - e r0), whose relative error is the square of the FP32 error
// (<= 2^-48) plus rounding; a denominator outside the FP32 normal range takes 1.0 / e.
__device__ __forceinline__ double h_recip(double e) {
    const float ef = __double2float_rn(e);
    const float af = fabsf(ef);
    if (!(af >= 1.1754944e-38f && af <= 3.0e38f)) return 1.0 / e;
    const double r0 = (double)__frcp_rn(ef);
    return fma(r0, fma(-e, r0, 1.0), r0);
}

__global__ void __launch_bounds__(256) h_stream_kernel(const cplx *__restrict__ Hc, int ni, int ns,
                                                       const double *__restrict__ eps_i,
                                                       const double *__restrict__ eps_s,
                                                       const int *__restrict__ irp_i, const int *__restrict__ irp_s,
                                                       const int *__restrict__ md, const int *__restrict__ msy,
                                                       int nsym, double eshift, double *e2part, double *sc2part) {
    __shared__ double sh[2][8];
    const int b = blockIdx.x, i = blockIdx.y + 1;
    const int64_t S = ns, I = ni;
    const int nab = ns - 1 - b;    // a = b + 1 .. ns - 1
    const int tot = i * nab;       // (j, a) pairs of this block
    const double cbi = eps_s[b] - eps_i[i] + eshift;
    const int irb = irp_s[b], iri = irp_i[i];
    const cplx *row1 = Hc + (b + 1) + S * (i + I * (int64_t)b);   // (a i|b j) = row1[a' + S I S j]
    const cplx *row2 = Hc + (b + 1) + S * I * (b + S * (int64_t)i);   // (a j|b i) = row2[a' + S j]
    double e2 = 0.0, sc2 = 0.0;
    for (int q = threadIdx.x; q < tot; q += blockDim.x) {
        const int j = q / nab, a1 = q - j * nab, a = b + 1 + a1;
        if (nsym > 1) {
            const int s1 = md[(irp_s[a] - 1) * nsym + iri - 1];
            const int s2 = md[(irb - 1) * nsym + irp_i[j] - 1];
            if (msy[(s1 - 1) * nsym + s2 - 1] != 1) continue;
        }
        const cplx x1 = __ldcs(row1 + a1 + S * I * S * (int64_t)j);
        const cplx x2 = __ldcs(row2 + a1 + S * (int64_t)j);
        const double vr = x1.x - x2.x, vi = x1.y - x2.y;
        const double a2 = fma(vr, vr, vi * vi);
        const double e = __ldg(eps_s + a) + (cbi - __ldg(eps_i + j));
        const double r = h_recip(e);
        const double t = a2 * r;
        e2 -= t;
        sc2 = fma(t, r, sc2);
    }
    // deterministic block reduction
    for (int o = 16; o > 0; o >>= 1) {
        e2 += __shfl_down_sync(0xffffffffu, e2, o);
        sc2 += __shfl_down_sync(0xffffffffu, sc2, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sh[0][wid] = e2; sh[1][wid] = sc2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) { x += sh[0][w]; y += sh[1][w]; }
        const int64_t blk = (int64_t)blockIdx.y * gridDim.x + blockIdx.x;
        e2part[blk] = x;
        sc2part[blk] = y;
    }
}

__global__ void zero2_kernel(double *a, double *b) {
    a[0] = 0.0;
    b[0] = 0.0;
}

int h_stream_blocks(int ni, int ns) { return (ni >= 2 && ns >= 2) ? (ns - 1) * (ni - 1) : 1; }

void launch_h_stream2(Context &c, const cplx *Hc, int ni, int ns, const double *eps_i, const double *eps_s,
                      const int *irp_i, const int *irp_s, const int *md, const int *msy, int nsym, double eshift,
                      double *e2part, double *sc2part) {
    if (ni < 2 || ns < 2) {   // no pair a > b, i > j
        zero2_kernel<<<1, 1, 0, c.stream>>>(e2part, sc2part);
    } else {
        h_stream_kernel<<<dim3((unsigned)(ns - 1), (unsigned)(ni - 1)), 256, 0, c.stream>>>(
            Hc, ni, ns, eps_i, eps_s, irp_i, irp_s, md, msy, nsym, eshift, e2part, sc2part);
    }
    DCG_LAUNCHED(c);
}

}  // namespace dcg

// ============================================================================ allocation-free H subspace
// dcg_solve_h for callers that cannot allocate device memory (a host that owns every
// device allocation through its own pool, a plug-in running under another runtime's
// allocator): the same H-subspace sum with one partial pair per inactive pair i > j,
// held in a file-scope device array instead of the context workspace.  The array is
// sized for at most DCG_H_NOALLOC_MAX_NINACT inactive spinors (8128 pairs, 127 KiB) and
// stays resident on every device that loads the library until the process exits.
namespace dcg {

constexpr int H_NOALLOC_MAX_NINACT = 128;
constexpr int H_NOALLOC_MAX_PAIRS = H_NOALLOC_MAX_NINACT * (H_NOALLOC_MAX_NINACT - 1) / 2;
// [0, P): e2 partial per pair; [P, 2P): sumc2 partial per pair; [2P, 2P+2): results
static __device__ __align__(256) double g_h_noalloc_scratch[2 * H_NOALLOC_MAX_PAIRS + 2];

// one block per inactive pair (i, j), i > j, ordered (1,0),(2,0),(2,1),...
__global__ void h_pair_kernel(const cplx *__restrict__ Hc, int ni, int ns, const double *__restrict__ eps_i,
                              const double *__restrict__ eps_s, const int *__restrict__ irp_i,
                              const int *__restrict__ irp_s, const int *__restrict__ md, const int *__restrict__ msy,
                              int nsym, double eshift, double *scratch) {
    __shared__ double sh[2][32];
    const int p = blockIdx.x;
    int i = 1, cnt = p;
    while (cnt >= i) { cnt -= i; i++; }
    const int j = cnt;
    const int64_t S = ns, I = ni;
    double e2 = 0.0, sc2 = 0.0;
    for (int64_t q = threadIdx.x; q < S * S; q += blockDim.x) {
        const int a = (int)(q % S), b = (int)(q / S);
        if (a <= b) continue;
        const int s1 = md[(irp_s[a] - 1) * nsym + irp_i[i] - 1];
        const int s2 = md[(irp_s[b] - 1) * nsym + irp_i[j] - 1];
        if (msy[(s1 - 1) * nsym + s2 - 1] != 1) continue;
        const cplx v = csub(Hc[a + S * (i + I * (b + S * (int64_t)j))], Hc[a + S * (j + I * (b + S * (int64_t)i))]);
        const double e = eps_s[a] + eps_s[b] - eps_i[i] - eps_i[j] + eshift;
        const double a2 = cabs2(v);
        e2 -= a2 / e;
        sc2 += a2 / (e * e);
    }
    for (int o = 16; o > 0; o >>= 1) {
        e2 += __shfl_down_sync(0xffffffffu, e2, o);
        sc2 += __shfl_down_sync(0xffffffffu, sc2, o);
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) { sh[0][wid] = e2; sh[1][wid] = sc2; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) { x += sh[0][w]; y += sh[1][w]; }
        scratch[p] = x;
        scratch[H_NOALLOC_MAX_PAIRS + p] = y;
    }
}

// fixed-order sum of the npair partials into the two result slots
__global__ void h_pair_final_kernel(double *scratch, int npair) {
    if (threadIdx.x != 0) return;
    double x = 0.0, y = 0.0;
    for (int p = 0; p < npair; p++) {
        x += scratch[p];
        y += scratch[H_NOALLOC_MAX_PAIRS + p];
    }
    scratch[2 * H_NOALLOC_MAX_PAIRS] = x;
    scratch[2 * H_NOALLOC_MAX_PAIRS + 1] = y;
}

}  // namespace dcg

extern "C" int dcg_solve_h_noalloc(const void *hclass, int32_t ninact, int32_t nsec, const double *eps_i,
                                   const double *eps_s, const int32_t *irp_i, const int32_t *irp_s,
                                   const int32_t *multb_d, const int32_t *multb_s, int32_t nsymrpa, double eshift,
                                   void *stream, double out[2]) {
    using namespace dcg;
    if (!out || ninact < 0 || nsec < 0 || nsymrpa < 1) return DCG_E_ARG;
    if (ninact > H_NOALLOC_MAX_NINACT) return DCG_E_ARG;   // beyond the static scratch
    out[0] = out[1] = 0.0;
    if (ninact < 2 || nsec < 2) return DCG_OK;              // no pair i > j or a > b
    if (!hclass || !eps_i || !eps_s || !irp_i || !irp_s || !multb_d || !multb_s) return DCG_E_ARG;
    // An error the caller left pending is not this call's: report it without clearing it, so
    // that the launch check below sees only these launches.
    if (cudaPeekAtLastError() != cudaSuccess) return DCG_E_CUDA;
    // The device address of the array in the context current now (the caller's device and
    // context; a context of its own, or one created again after cudaDeviceReset, has its own
    // copy of the array), looked up on every call.
    double *scratch = nullptr;
    if (cudaGetSymbolAddress((void **)&scratch, g_h_noalloc_scratch) != cudaSuccess || !scratch) return DCG_E_CUDA;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int npair = ninact * (ninact - 1) / 2;
    h_pair_kernel<<<npair, 256, 0, st>>>(static_cast<const cplx *>(hclass), ninact, nsec, eps_i, eps_s, irp_i, irp_s,
                                         multb_d, multb_s, nsymrpa, eshift, scratch);
    h_pair_final_kernel<<<1, 32, 0, st>>>(scratch, npair);
    if (cudaGetLastError() != cudaSuccess) return DCG_E_CUDA;
    if (cudaMemcpyAsync(out, scratch + 2 * H_NOALLOC_MAX_PAIRS, 2 * sizeof(double), cudaMemcpyDeviceToHost, st) !=
        cudaSuccess)
        return DCG_E_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return DCG_E_CUDA;
    return DCG_OK;
}
