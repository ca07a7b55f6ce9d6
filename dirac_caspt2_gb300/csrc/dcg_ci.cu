// Determinant-space kernels: CASCI Hamiltonian, one-electron excitation gathers that
// turn the reference's dimN_density loops into GEMM operands, and the determinant
// overlap matrix of the CI rotation.
//
// Bit t of a determinant bit string <-> active spinor t (one_e_exct.F90:30-46).
// E_{ca}|I> = (-1)^phase |J>, J = I - bit a + bit c, with
// phase = popcount(I & bits above a) + popcount((I - bit a) & bits above c)
// (one_e_exct.F90:38-46).  The full N-electron space is every nelec-of-nact bit string in
// increasing integer (colex) order, so the position of a string is its combinatorial
// number sum_k C(p_k, k+1) over its set bits p_0 < p_1 < ...
#include "dcg_common.cuh"
#include "dcg_kernels.cuh"

namespace dcg {

__constant__ int64_t c_binom[65][65];

namespace {
struct BinomTable {
    int64_t t[65][65];
    BinomTable() {
        for (int n = 0; n <= 64; n++) {
            t[n][0] = 1;
            for (int k = 1; k <= 64; k++) t[n][k] = (n == 0) ? 0 : t[n - 1][k - 1] + (k <= n - 1 ? t[n - 1][k] : 0);
        }
    }
};
}  // namespace

// The table is the same for every context; contexts created from several host threads write
// identical bytes (the static is initialised once, thread-safely).
void upload_binomials(Context &c) {
    static const BinomTable tab;
    DCG_CUDA(cudaMemcpyToSymbolAsync(c_binom, tab.t, sizeof(tab.t), 0, cudaMemcpyHostToDevice, c.stream));
}

__device__ __forceinline__ int64_t colex_rank(uint64_t I) {
    int64_t r = 0;
    int k = 1;
    while (I) {
        int p = __ffsll((long long)I) - 1;
        r += c_binom[p][k];
        k++;
        I &= I - 1;
    }
    return r;
}

// E_{ca} on bit string I: returns false when the result vanishes.
__device__ __forceinline__ bool exct(uint64_t I, int c, int a, int na, uint64_t &J, int &phase) {
    const uint64_t ba = 1ull << a, bc = 1ull << c;
    if (c == a) {
        if (!(I & ba)) return false;
        J = I;
        phase = 0;
        return true;
    }
    if (!(I & ba) || (I & bc)) return false;
    J = I - ba + bc;
    const uint64_t full = (na >= 64) ? ~0ull : ((1ull << na) - 1ull);
    const uint64_t above_a = full & ~((ba << 1) - 1ull);
    const uint64_t above_c = full & ~((bc << 1) - 1ull);
    phase = __popcll(I & above_a) + __popcll((I - ba) & above_c);
    return true;
}

__device__ __forceinline__ int64_t find_sorted(const uint64_t *__restrict__ v, int64_t n, uint64_t key) {
    int64_t lo = 0, hi = n - 1;
    while (lo <= hi) {
        int64_t mid = (lo + hi) >> 1;
        uint64_t x = v[mid];
        if (x == key) return mid;
        if (x < key) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

// ------------------------------------------------------------------------- CASCI matrix
// One block per determinant row i; writes H(i,j) and H(j,i)=conj for connected j > i
// and the diagonal (casmat.F90:3-222).  g: inttw, (nmoc)^4 column-major.
__global__ void casmat_kernel(int ni, int na, int ne, const uint64_t *__restrict__ dets, int ndet,
                              const cplx *__restrict__ h, int nmo, const cplx *__restrict__ g, cplx *H) {
    __shared__ int occ[64], vir[64];
    __shared__ double red[32];
    const int i = blockIdx.x;
    const uint64_t I = dets[i];
    const int nmoc = ni + na;
    if (threadIdx.x == 0) {
        int no = 0, nv = 0;
        for (int t = 0; t < na; t++) {
            if ((I >> t) & 1ull) occ[no++] = t;
            else vir[nv++] = t;
        }
    }
    __syncthreads();
    const int nv = na - ne;
    const int nocc = ni + ne;   // global occupied list: inactive then active occupied
#define GIDX(p, q, r, s) ((int64_t)(p) + (int64_t)nmoc * ((q) + (int64_t)nmoc * ((r) + (int64_t)nmoc * (s))))
#define OCCG(x) ((x) < ni ? (x) : ni + occ[(x) - ni])
    // diagonal: sum_r Re h_rr + sum_{r<s} Re[(rr|ss) - (rs|sr)]
    double acc = 0.0;
    const int64_t npair = (int64_t)nocc * nocc;
    for (int64_t q = threadIdx.x; q < npair; q += blockDim.x) {
        int x = (int)(q % nocc), y = (int)(q / nocc);
        if (y <= x) continue;
        int r = OCCG(x), s = OCCG(y);
        acc += g[GIDX(r, r, s, s)].x - g[GIDX(r, s, s, r)].x;
    }
    for (int x = threadIdx.x; x < nocc; x += blockDim.x) {
        int r = OCCG(x);
        acc += h[r + (int64_t)nmo * r].x;
    }
    {
        int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if (lane == 0) red[wid] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double s = 0.0;
            for (int w = 0; w < (int)((blockDim.x + 31) >> 5); w++) s += red[w];
            H[i + (int64_t)ndet * i] = mk(s, 0.0);
        }
    }
    // singles
    const int nsing = ne * nv;
    for (int q = threadIdx.x; q < nsing; q += blockDim.x) {
        int ro = occ[q / nv], av = vir[q % nv];
        uint64_t J;
        int ph;
        if (!exct(I, av, ro, na, J, ph)) continue;
        int64_t j = find_sorted(dets, ndet, J);
        if (j <= i) continue;
        const int ir = ni + ro, ia = ni + av;
        cplx v = h[ir + (int64_t)nmo * ia];
        for (int x = 0; x < nocc; x++) {
            int s = OCCG(x);
            v = cadd(v, g[GIDX(ir, ia, s, s)]);
            v = csub(v, g[GIDX(ir, s, s, ia)]);
        }
        if (ph & 1) v = mk(-v.x, -v.y);
        H[i + (int64_t)ndet * j] = v;
        H[j + (int64_t)ndet * i] = cconj(v);
    }
    // doubles
    const int npo = ne * (ne - 1) / 2, npv = nv * (nv - 1) / 2;
    const int64_t ndbl = (int64_t)npo * npv;
    for (int64_t q = threadIdx.x; q < ndbl; q += blockDim.x) {
        int po = (int)(q / npv), pv = (int)(q % npv);
        int x = 0, y = 0;
        {
            int cnt = po;
            for (x = 0; x < ne; x++) {
                int rem = ne - 1 - x;
                if (cnt < rem) { y = x + 1 + cnt; break; }
                cnt -= rem;
            }
        }
        int u = 0, w2 = 0;
        {
            int cnt = pv;
            for (u = 0; u < nv; u++) {
                int rem = nv - 1 - u;
                if (cnt < rem) { w2 = u + 1 + cnt; break; }
                cnt -= rem;
            }
        }
        const int r_ = occ[x], s_ = occ[y], a_ = vir[u], b_ = vir[w2];
        uint64_t J1, J2;
        int p1, p2;
        if (!exct(I, a_, r_, na, J1, p1)) continue;
        if (!exct(J1, b_, s_, na, J2, p2)) continue;
        int64_t j = find_sorted(dets, ndet, J2);
        if (j <= i) continue;
        const int ir = ni + r_, is = ni + s_, ia = ni + a_, ib = ni + b_;
        cplx v = csub(g[GIDX(ir, ia, is, ib)], g[GIDX(ir, ib, is, ia)]);
        if ((p1 + p2) & 1) v = mk(-v.x, -v.y);
        H[i + (int64_t)ndet * j] = v;
        H[j + (int64_t)ndet * i] = cconj(v);
    }
#undef OCCG
#undef GIDX
}

// ------------------------------------------------------------------------- sparse CASCI matrix
// The same Slater-Condon elements (casmat.F90:3-222), as a CSR matrix for the Davidson route:
// row i holds its diagonal and every single and double excitation of det i that lies in the
// CI space (RAS restrictions included).  Candidates of a row: q < ne nv singles, then the
// ne(ne-1)/2 x nv(nv-1)/2 doubles.  An element H(i, j) with j > i is computed from det i as
// the dense kernel does; one with j < i is conj(H(j, i)) computed from det j by the same
// arithmetic in the same order, so the matrix is Hermitian to the bit (the dense kernel
// mirrors its upper triangle the same way).
struct CsrRow {
    int occ[64], vir[64];
};

// <single excitation av <- ro of the source determinant S> (S holds ro, not av): h plus the
// sum over S's occupied spinors (inactive, then active in increasing order), signed by the
// excitation's phase.
__device__ cplx single_elem(int ni, int na, const cplx *__restrict__ h, int nmo, const cplx *__restrict__ g,
                            uint64_t S, int ro, int av) {
    const int nmoc = ni + na;
#define GIDX(p, q_, r, s) ((int64_t)(p) + (int64_t)nmoc * ((q_) + (int64_t)nmoc * ((r) + (int64_t)nmoc * (s))))
    uint64_t J;
    int ph;
    exct(S, av, ro, na, J, ph);
    const int ir = ni + ro, ia = ni + av;
    cplx v = h[ir + (int64_t)nmo * ia];
    for (int k = 0; k < ni; k++) {
        v = cadd(v, g[GIDX(ir, ia, k, k)]);
        v = csub(v, g[GIDX(ir, k, k, ia)]);
    }
    for (uint64_t B = S; B; B &= B - 1) {
        const int s2 = ni + __ffsll((long long)B) - 1;
        v = cadd(v, g[GIDX(ir, ia, s2, s2)]);
        v = csub(v, g[GIDX(ir, s2, s2, ia)]);
    }
    if (ph & 1) v = mk(-v.x, -v.y);
    return v;
}

// <double excitation a <- r, b <- s of S> (r < s occupied, a < b empty).
__device__ cplx double_elem(int ni, int na, const cplx *__restrict__ g, uint64_t S, int r_, int s_, int a_, int b_) {
    const int nmoc = ni + na;
    uint64_t J1, J2;
    int p1, p2;
    exct(S, a_, r_, na, J1, p1);
    exct(J1, b_, s_, na, J2, p2);
    const int ir = ni + r_, is = ni + s_, ia = ni + a_, ib = ni + b_;
    cplx v = csub(g[GIDX(ir, ia, is, ib)], g[GIDX(ir, ib, is, ia)]);
    if ((p1 + p2) & 1) v = mk(-v.x, -v.y);
    return v;
#undef GIDX
}

// Candidate q of row i (determinant I): false when the excitation vanishes or leaves the CI
// space; else its column and (WANT_VAL) its element.
template <bool WANT_VAL>
__device__ bool casmat_candidate(int ni, int na, int ne, const uint64_t *__restrict__ dets, int ndet,
                                 const cplx *__restrict__ h, int nmo, const cplx *__restrict__ g, int64_t i,
                                 uint64_t I, const CsrRow &rw, int64_t q, int64_t &jout, cplx &vout) {
    const int nv = na - ne;
    const int64_t nsing = (int64_t)ne * nv;
    if (q < nsing) {
        const int ro = rw.occ[q / nv], av = rw.vir[q % nv];
        uint64_t J;
        int ph;
        if (!exct(I, av, ro, na, J, ph)) return false;
        const int64_t j = find_sorted(dets, ndet, J);
        if (j < 0) return false;
        jout = j;
        if (WANT_VAL) vout = j > i ? single_elem(ni, na, h, nmo, g, I, ro, av) : cconj(single_elem(ni, na, h, nmo, g, J, av, ro));
        return true;
    }
    q -= nsing;
    const int npv = nv * (nv - 1) / 2;
    const int po = (int)(q / npv), pv = (int)(q % npv);
    int x = 0, y = 0, u = 0, w2 = 0;
    {
        int cnt = po;
        for (x = 0; x < ne; x++) {
            const int rem = ne - 1 - x;
            if (cnt < rem) {
                y = x + 1 + cnt;
                break;
            }
            cnt -= rem;
        }
    }
    {
        int cnt = pv;
        for (u = 0; u < nv; u++) {
            const int rem = nv - 1 - u;
            if (cnt < rem) {
                w2 = u + 1 + cnt;
                break;
            }
            cnt -= rem;
        }
    }
    const int r_ = rw.occ[x], s_ = rw.occ[y], a_ = rw.vir[u], b_ = rw.vir[w2];
    uint64_t J1, J2;
    int p1, p2;
    if (!exct(I, a_, r_, na, J1, p1)) return false;
    if (!exct(J1, b_, s_, na, J2, p2)) return false;
    const int64_t j = find_sorted(dets, ndet, J2);
    if (j < 0) return false;
    jout = j;
    // from det j the occupied pair is (a, b) and the empty pair (r, s), both increasing
    if (WANT_VAL) vout = j > i ? double_elem(ni, na, g, I, r_, s_, a_, b_) : cconj(double_elem(ni, na, g, J2, a_, b_, r_, s_));
    return true;
}

__device__ void casmat_row_setup(int na, uint64_t I, CsrRow &rw) {
    if (threadIdx.x == 0) {
        int no = 0, nv = 0;
        for (int t = 0; t < na; t++) {
            if ((I >> t) & 1ull) rw.occ[no++] = t;
            else rw.vir[nv++] = t;
        }
    }
    __syncthreads();
}

// Diagonal of row i (block reduction), as casmat_kernel.
__device__ double casmat_diag(int ni, int na, int ne, const cplx *__restrict__ h, int nmo, const cplx *__restrict__ g,
                              const CsrRow &rw, double *red) {
    const int nmoc = ni + na, nocc = ni + ne;
#define GIDX(p, q_, r, s) ((int64_t)(p) + (int64_t)nmoc * ((q_) + (int64_t)nmoc * ((r) + (int64_t)nmoc * (s))))
#define OCCG(x) ((x) < ni ? (x) : ni + rw.occ[(x) - ni])
    double acc = 0.0;
    const int64_t npair = (int64_t)nocc * nocc;
    for (int64_t q = threadIdx.x; q < npair; q += blockDim.x) {
        const int x = (int)(q % nocc), y = (int)(q / nocc);
        if (y <= x) continue;
        const int r = OCCG(x), s2 = OCCG(y);
        acc += g[GIDX(r, r, s2, s2)].x - g[GIDX(r, s2, s2, r)].x;
    }
    for (int x = threadIdx.x; x < nocc; x += blockDim.x) {
        const int r = OCCG(x);
        acc += h[r + (int64_t)nmo * r].x;
    }
#undef OCCG
#undef GIDX
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) red[wid] = acc;
    __syncthreads();
    double s = 0.0;
    for (int w = 0; w < (int)((blockDim.x + 31) >> 5); w++) s += red[w];
    __syncthreads();
    return s;
}

__global__ void __launch_bounds__(256) casmat_csr_count_kernel(int ni, int na, int ne, const uint64_t *__restrict__ dets,
                                                               int ndet, const cplx *__restrict__ h, int nmo,
                                                               const cplx *__restrict__ g, int64_t *counts) {
    __shared__ CsrRow rw;
    __shared__ int64_t red[8];
    const int i = blockIdx.x;
    const uint64_t I = dets[i];
    casmat_row_setup(na, I, rw);
    const int nv = na - ne;
    const int64_t ncand = (int64_t)ne * nv + (int64_t)(ne * (ne - 1) / 2) * (nv * (nv - 1) / 2);
    int64_t cnt = 0;
    for (int64_t q = threadIdx.x; q < ncand; q += blockDim.x) {
        int64_t j;
        cplx v;
        cnt += casmat_candidate<false>(ni, na, ne, dets, ndet, h, nmo, g, i, I, rw, q, j, v) ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 1;   // the diagonal
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        counts[i] = t;
    }
}

__global__ void __launch_bounds__(256) casmat_csr_fill_kernel(int ni, int na, int ne, const uint64_t *__restrict__ dets,
                                                              int ndet, const cplx *__restrict__ h, int nmo,
                                                              const cplx *__restrict__ g, const int64_t *rowptr,
                                                              int *cols, cplx *vals, double *hdiag) {
    __shared__ CsrRow rw;
    __shared__ double red[8];
    __shared__ int wsum[8];
    __shared__ int64_t run;
    const int i = blockIdx.x;
    const uint64_t I = dets[i];
    casmat_row_setup(na, I, rw);
    const double dg = casmat_diag(ni, na, ne, h, nmo, g, rw, red);
    if (threadIdx.x == 0) {
        cols[rowptr[i]] = i;
        vals[rowptr[i]] = mk(dg, 0.0);
        hdiag[i] = dg;
        run = rowptr[i] + 1;
    }
    __syncthreads();
    const int nv = na - ne;
    const int64_t ncand = (int64_t)ne * nv + (int64_t)(ne * (ne - 1) / 2) * (nv * (nv - 1) / 2);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int64_t q0 = 0; q0 < ncand; q0 += blockDim.x) {
        const int64_t q = q0 + threadIdx.x;
        int64_t j = 0;
        cplx v = mk(0.0, 0.0);
        const bool kept = q < ncand && casmat_candidate<true>(ni, na, ne, dets, ndet, h, nmo, g, i, I, rw, q, j, v);
        const unsigned bal = __ballot_sync(0xffffffffu, kept);
        if (lane == 0) wsum[warp] = __popc(bal);
        __syncthreads();
        int before = 0, total = 0;
        for (int w = 0; w < nw; w++) {
            if (w < warp) before += wsum[w];
            total += wsum[w];
        }
        before += __popc(bal & ((1u << lane) - 1u));
        if (kept) {
            cols[run + before] = (int)j;
            vals[run + before] = v;
        }
        __syncthreads();
        if (threadIdx.x == 0) run += total;
        __syncthreads();
    }
}

void build_casmat_csr(Context &c, const uint64_t *dets, int ndet, const cplx *h, const cplx *g, CsrMatrix &m) {
    if (c.na > 64) throw Error{DCG_E_ARG, "casmat: more than 64 active spinors"};
    int64_t *counts = wsget<int64_t>(c, "csr.cnt", (size_t)ndet + 1);
    casmat_csr_count_kernel<<<ndet, 256, 0, c.stream>>>(c.ni, c.na, c.ne, dets, ndet, h, c.nmo, g, counts);
    DCG_LAUNCHED(c);
    std::vector<int64_t> hc(ndet), rp((size_t)ndet + 1, 0);
    DCG_CUDA(cudaMemcpyAsync(hc.data(), counts, sizeof(int64_t) * ndet, cudaMemcpyDeviceToHost, c.stream));
    DCG_CUDA(cudaStreamSynchronize(c.stream));
    for (int i = 0; i < ndet; i++) rp[i + 1] = rp[i] + hc[i];
    m.n = ndet;
    m.nnz = rp[ndet];
    m.rowptr = wsget<int64_t>(c, "csr.rp", (size_t)ndet + 1);
    DCG_CUDA(cudaMemcpyAsync(m.rowptr, rp.data(), sizeof(int64_t) * (ndet + 1), cudaMemcpyHostToDevice, c.stream));
    m.cols = wsget<int>(c, "csr.col", (size_t)m.nnz + 1);
    m.vals = wsget<cplx>(c, "csr.val", (size_t)m.nnz + 1);
    m.diag = wsget<double>(c, "csr.diag", (size_t)ndet + 1);
    casmat_csr_fill_kernel<<<ndet, 256, 0, c.stream>>>(c.ni, c.na, c.ne, dets, ndet, h, c.nmo, g, m.rowptr, m.cols,
                                                        m.vals, m.diag);
    DCG_LAUNCHED(c);
}

void launch_casmat(Context &c, const uint64_t *dets, int ndet, const cplx *h, const cplx *g, cplx *H) {
    DCG_CUDA(cudaMemsetAsync(H, 0, sizeof(cplx) * (size_t)ndet * ndet, c.stream));
    casmat_kernel<<<ndet, 256, 0, c.stream>>>(c.ni, c.na, c.ne, dets, ndet, h, c.nmo, g, H);
    DCG_LAUNCHED(c);
}

// ------------------------------------------------------------------------- excitation gathers
// out[K, p + na*q, v] = (E_pq x_v)[K] over the full N-space (M strings, colex order):
// the source string is L = E_qp K and the sign is that of E_qp acting on K.
// x: M x nv (ldx = M); out: M x na^2 x nv.
__global__ void apply_E_kernel(int na, int64_t M, const uint64_t *__restrict__ full, const cplx *__restrict__ x,
                               int nv, cplx *out) {
    const int64_t K = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int pq = blockIdx.y;
    if (K >= M) return;
    const int p = pq % na, q = pq / na;
    const uint64_t IK = full[K];
    uint64_t L;
    int ph;
    const int64_t na2 = (int64_t)na * na;
    if (!exct(IK, q, p, na, L, ph)) {
        for (int v = 0; v < nv; v++) out[K + M * (pq + na2 * v)] = mk(0.0, 0.0);
        return;
    }
    const int64_t l = colex_rank(L);
    for (int v = 0; v < nv; v++) {
        cplx val = x[l + M * v];
        if (ph & 1) val = mk(-val.x, -val.y);
        out[K + M * (pq + na2 * v)] = val;
    }
}

void launch_apply_E(Context &c, int na, int64_t M, const uint64_t *full, const cplx *x, int nv, cplx *out) {
    const int64_t na2 = (int64_t)na * na;
    for (int64_t p0 = 0; p0 < na2; p0 += 65535) {
        (void)p0;
    }
    dim3 grid(grid1d(M, 128), (unsigned)na2);
    apply_E_kernel<<<grid, 128, 0, c.stream>>>(na, M, full, x, nv, out);
    DCG_LAUNCHED(c);
}

// Gram factor of the A and C overlap matrices.  Column j of G holds, over the determinants of
// the (nelec +- 1)-electron space (colex order, dets_p), the vector
//   create = 1 (subspace A): a_x^+ E_yz |0>     create = 0 (subspace C): a_x E_yz |0>
// with (x, y, z) = ind[3j..3j+2] and E_yz|0> taken from Y (column y + na z, M rows, the
// nelec-electron full space).  Sign convention of the CI code: a creation or annihilation of
// orbital x carries (-1)^(occupied orbitals above x).  With it, S = G^H G and B = G^H D G
// where D is the active Fock operator, diagonal over the determinants of dets_p.
__global__ void gram_kernel(int na, int64_t Mp, const uint64_t *__restrict__ dets_p, int64_t M,
                            const cplx *__restrict__ Y, const int *__restrict__ ind, int dimn, int create,
                            cplx *G) {
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int j = blockIdx.y;
    if (r >= Mp || j >= dimn) return;
    const int x = ind[3 * j], y = ind[3 * j + 1], z = ind[3 * j + 2];
    const uint64_t J = dets_p[r];
    const uint64_t bit = 1ull << x;
    cplx val = mk(0.0, 0.0);
    const bool has = (J & bit) != 0;
    if (create ? has : !has) {
        const uint64_t I = create ? (J & ~bit) : (J | bit);   // nelec-electron source determinant
        const uint64_t above = I & ~((bit << 1) - 1);
        val = Y[colex_rank(I) + M * (int64_t)(y + na * z)];
        if (__popcll(above) & 1) val = mk(-val.x, -val.y);
    }
    G[r + Mp * (int64_t)j] = val;
}

void launch_gram(Context &c, int na, int64_t Mp, const uint64_t *dets_p, int64_t M, const cplx *Y, const int *ind,
                 int dimn, int create, cplx *G) {
    dim3 grid(grid1d(Mp, 128), (unsigned)dimn);
    gram_kernel<<<grid, 128, 0, c.stream>>>(na, Mp, dets_p, M, Y, ind, dimn, create, G);
    DCG_LAUNCHED(c);
}

// A(i, j) *= s[i] (column-major, lda)
__global__ void scale_rows_kernel(int m, int n, cplx *A, int64_t lda, const double *__restrict__ s, int soff, int inv) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)m * n) return;
    const int i = (int)(idx % m), j = (int)(idx / m);
    const double f = inv ? 1.0 / s[soff + i] : s[soff + i];
    cplx &a = A[i + (int64_t)j * lda];
    a = mk(a.x * f, a.y * f);
}

void launch_scale_rows(Context &c, int m, int n, cplx *A, int64_t lda, const double *s, int soff, bool inv) {
    if ((int64_t)m * n == 0) return;
    scale_rows_kernel<<<grid1d((int64_t)m * n, 256), 256, 0, c.stream>>>(m, n, A, lda, s, soff, inv ? 1 : 0);
    DCG_LAUNCHED(c);
}

// psi_t[K] = psi[K] * sum_{w in K} eps_act[w]  (Fock operator of the active space acting
// on |0>, the E_ww factor of the reference's dim(n+1)_density(..., w, w) calls)
__global__ void occ_energy_kernel(int na, int64_t M, const uint64_t *__restrict__ full, const double *__restrict__ eps_act,
                                  const cplx *__restrict__ psi, cplx *psit) {
    const int64_t K = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (K >= M) return;
    uint64_t I = full[K];
    double s = 0.0;
    while (I) {
        int t = __ffsll((long long)I) - 1;
        s += eps_act[t];
        I &= I - 1;
    }
    psit[K] = cscale(psi[K], s);
}

void launch_occ_energy(Context &c, int na, int64_t M, const uint64_t *full, const double *eps_act, const cplx *psi,
                       cplx *psit) {
    occ_energy_kernel<<<grid1d(M, 256), 256, 0, c.stream>>>(na, M, full, eps_act, psi, psit);
    DCG_LAUNCHED(c);
}

__global__ void embed_kernel(int ndet, const int64_t *__restrict__ pos, const cplx *__restrict__ cvec, cplx *psi) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ndet) psi[pos[i]] = cvec[i];
}

void launch_embed(Context &c, int ndet, const int64_t *pos, const cplx *cvec, cplx *psi, int64_t M) {
    DCG_CUDA(cudaMemsetAsync(psi, 0, sizeof(cplx) * M, c.stream));
    embed_kernel<<<grid1d(ndet, 256), 256, 0, c.stream>>>(ndet, pos, cvec, psi);
    DCG_LAUNCHED(c);
}

// ------------------------------------------------------------------------- CI rotation
// ds(a,b) = det(U[occ_a, occ_b]) (trac.F90:76-156, sdet.F90:58-110); LU with partial pivoting.
constexpr int MAXE = 20;
__global__ void detsc_kernel(int ne, int na, const uint64_t *__restrict__ dets, int ndet, const cplx *__restrict__ U,
                             cplx *ds) {
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)ndet * ndet) return;
    const int a = (int)(idx % ndet), b = (int)(idx / ndet);
    int oa[MAXE], ob[MAXE];
    {
        uint64_t I = dets[a];
        int k = 0;
        while (I) { oa[k++] = __ffsll((long long)I) - 1; I &= I - 1; }
        I = dets[b];
        k = 0;
        while (I) { ob[k++] = __ffsll((long long)I) - 1; I &= I - 1; }
    }
    cplx m[MAXE * MAXE];
    for (int r = 0; r < ne; r++)
        for (int s = 0; s < ne; s++) m[r + ne * s] = U[oa[r] + (int64_t)na * ob[s]];
    cplx det = mk(1.0, 0.0);
    for (int k = 0; k < ne; k++) {
        int p = k;
        double best = cabs2(m[k + ne * k]);
        for (int r = k + 1; r < ne; r++) {
            double v = cabs2(m[r + ne * k]);
            if (v > best) { best = v; p = r; }
        }
        if (best == 0.0) { det = mk(0.0, 0.0); break; }
        if (p != k) {
            for (int s = 0; s < ne; s++) {
                cplx t = m[k + ne * s];
                m[k + ne * s] = m[p + ne * s];
                m[p + ne * s] = t;
            }
            det = mk(-det.x, -det.y);
        }
        cplx piv = m[k + ne * k];
        det = cmul(det, piv);
        cplx inv = cdiv(mk(1.0, 0.0), piv);
        for (int r = k + 1; r < ne; r++) {
            cplx f = cmul(m[r + ne * k], inv);
            for (int s = k + 1; s < ne; s++) m[r + ne * s] = csub(m[r + ne * s], cmul(f, m[k + ne * s]));
        }
    }
    ds[a + (int64_t)ndet * b] = det;
}

void launch_detsc(Context &c, const uint64_t *dets, int ndet, const cplx *Uact, cplx *ds) {
    if (c.ne > MAXE) throw Error{DCG_E_ARG, "nelec above the CI-rotation kernel limit"};
    int64_t n2 = (int64_t)ndet * ndet;
    detsc_kernel<<<grid1d(n2, 128), 128, 0, c.stream>>>(c.ne, c.na, dets, ndet, Uact, ds);
    DCG_LAUNCHED(c);
}

}  // namespace dcg
