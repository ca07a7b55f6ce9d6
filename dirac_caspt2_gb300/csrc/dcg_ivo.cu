// Improved virtual orbitals (r4divo.F90:80-93, fockivo.F90:44-270): the Fock matrix of the
// secondary spinors for the state with one electron removed from the HOMO spinors, and its
// eigenvectors per abelian irrep block.
//
// The IVO orbitals written back to DFPCMO are ZHEEV's eigenvectors (diag.F90:66-128), and the
// sign of each is what that algorithm leaves, so the blocks are diagonalised by the LAPACK
// ZHEEV algorithm itself (dcg_zheev.cuh), one CTA per block.
#include <algorithm>
#include <vector>

#include "dcg_common.cuh"
#include "dcg_zheev.cuh"

namespace dcg {

namespace {

// one CTA per job
__global__ void __launch_bounds__(zheev_detail::kZheevThreads) zheev_lapack_kernel(const zheev_detail::ZheevJob *__restrict__ jobs,
                                                                                 int *status) {
    const int st = zheev_detail::zheev_cta(jobs[blockIdx.x]);
    if (threadIdx.x == 0) status[blockIdx.x] = st;
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
    std::vector<zheev_detail::ZheevJob> jobs(nb);
    for (int b = 0; b < nb; b++) {
        const int n = (int)blocks[b].size();
        const std::string tg = "#" + std::to_string(b);
        zheev_detail::ZheevJob &J = jobs[b];
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
    zheev_detail::ZheevJob *jd = upload(c, "ivo.jobs", jobs);
    int *st = wsget<int>(c, "ivo.st", nb);
    DCG_CUDA(cudaMemsetAsync(st, 0, sizeof(int) * nb, c.stream));
    zheev_lapack_kernel<<<nb, zheev_detail::kZheevThreads, 0, c.stream>>>(jd, st);
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
