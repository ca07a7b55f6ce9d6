// C ABI and orchestration of the CASCI / CASPT2 hot path on one GB300.
//
// The call sequence mirrors the reference drivers:
//   dcg_set_system : readint2_casci + divide_2_elec_integral_into_subspaces
//                    (module_2integrals.F90:26-588, divide_2_elec...F90:3-409) as one
//                    device scatter of the MDCINTNEW records into dense class tensors;
//   dcg_casci      : casci (casci.F90:3-163) = search_cas_configuration + casmat + cdiag;
//   dcg_caspt2     : r4dcaspt2_tra (r4dcaspt2_tra.F90:77-445) = fockcasci, fockdiag (+tracic),
//                    calce0, intra_1/2/3 and solve_A..H_subspace.
// Every dimN_density element of the reference is taken from dense density tensors
// computed once per solve by GEMMs over excited CI vectors (see rdm_build below).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "dcg_common.cuh"
#include "dcg_kernels.cuh"

struct dcg_ctx {
    dcg::Context c;
};

namespace dcg {

// ------------------------------------------------------------------------- host helpers
static std::vector<uint64_t> gosper_all(int na, int ne) {
    std::vector<uint64_t> out;
    if (ne < 0 || ne > na || na > 64) return out;
    if (ne == 0) {
        out.push_back(0);
        return out;
    }
    uint64_t cur = (ne == 64) ? ~0ull : ((1ull << ne) - 1ull);
    const uint64_t lim = (na == 64) ? 0 : (1ull << na);
    while (true) {
        out.push_back(cur);
        uint64_t t = (cur | (cur - 1)) + 1;
        uint64_t nxt = t | ((((t & (~t + 1)) / (cur & (~cur + 1))) >> 1) - 1);
        if (nxt <= cur) break;
        if (na < 64 && nxt >= lim) break;
        cur = nxt;
    }
    return out;
}

// search_cas_configuration.F90:91-110 + ras_det_check.F90:1-59
static bool ras_ok(const Context &c, uint64_t I) {
    if (c.ras1) {
        const uint64_t m = (c.ras1 >= 64) ? ~0ull : ((1ull << c.ras1) - 1ull);
        const int n1 = __builtin_popcountll(I & m);
        if (!(c.ras1 - c.ras1_max_hole <= n1 && n1 <= c.ras1 - c.min_hole_ras1)) return false;
    }
    if (c.ras3) {
        const int sh = c.ras1 + c.ras2;
        const uint64_t hi = (sh >= 64) ? 0 : ((I >> sh) << sh);
        const int n3 = __builtin_popcountll(I & hi);
        if (!(n3 <= c.ras3_max_elec && c.min_elec_ras3 <= n3)) return false;
    }
    return true;
}

// cas_configuration_totsym (search_cas_configuration.F90:112-149)
static int det_totsym(const Context &c, uint64_t I) {
    if (c.nsym == 1) return 1;
    int ret = 1, ielec = 0;
    for (int t = 0; t < c.na; t++) {
        if (!((I >> t) & 1ull)) continue;
        ielec++;
        const int jsym = c.irpamo[c.ni + t];
        if (ielec % 2 == 1) {
            ret = c.multb_ds[(jsym - 1) * c.nsym + (ret - 1)];
        } else {
            const int partner = (jsym % 2 == 1) ? jsym + 1 : jsym - 1;
            ret = c.multb_d[(partner - 1) * c.nsym + (ret - 1)];
        }
    }
    if (ielec % 2 == 0) ret += c.nsym;
    return ret;
}

static std::vector<uint64_t> enumerate_ci(const Context &c) {
    std::vector<uint64_t> out;
    for (uint64_t I : gosper_all(c.na, c.ne))
        if (ras_ok(c, I) && (c.nsym == 1 || det_totsym(c, I) == c.totsym)) out.push_back(I);
    return out;
}


// Stage names double as NVTX range names, so a profiler can select one stage's launches.
static const char *const kStageName[ST_COUNT] = {"ints", "casci_matrix", "casci_eig", "fock", "ci_rotation",
                                                 "rdm", "transformation", "A", "B", "C", "D", "E", "F", "G", "H",
                                                 "AC", "BDEFG"};
static void stage_begin(Context &c, int st) {
    nvtxRangePushA(kStageName[st]);
    DCG_CUDA(cudaEventRecord(c.ev[st], c.stream));
}
static void stage_end(Context &c, int st) {
    nvtxRangePop();
    DCG_CUDA(cudaEventRecord(c.ev[ST_COUNT], c.stream));
    DCG_CUDA(cudaEventSynchronize(c.ev[ST_COUNT]));
    float ms = 0.f;
    DCG_CUDA(cudaEventElapsedTime(&ms, c.ev[st], c.ev[ST_COUNT]));
    c.stage_ms[st] += ms;
}

// ------------------------------------------------------------------------- device state
struct DevSystem {
    cplx *h = nullptr;
    cplx *inttw = nullptr;
    ClassTensor cls[CL_COUNT];
    int *irp = nullptr;
    int *md = nullptr, *msy = nullptr;
    double *eps = nullptr;
    cplx *c0 = nullptr;   // CASCI vector of selectroot
    int ndet = 0;
    uint64_t *dets = nullptr;
};

static DevSystem &dev(Context &c) {
    if (!c.dev_state) c.dev_state = new DevSystem();
    return *static_cast<DevSystem *>(c.dev_state);
}

__global__ void pack_cplx_kernel(const double *re, const double *im, int64_t n, cplx *out) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = mk(re[i], im ? im[i] : 0.0);
}

// ------------------------------------------------------------------------- set_system
static void set_system(Context &c, const dcg_system *s) {
    if (!s) throw Error{DCG_E_ARG, "system is NULL"};
    if (s->ninact < 0 || s->nact < 0 || s->nsec < 0 || s->nelec < 0 || s->nelec > s->nact)
        throw Error{DCG_E_ARG, "bad ninact/nact/nsec/nelec"};
    if (s->nact > 63) throw Error{DCG_E_ARG, "nact above 63 is not supported (64-bit determinant strings)"};
    if (s->nmo < s->ninact + s->nact + s->nsec) throw Error{DCG_E_ARG, "nmo < ninact + nact + nsec"};
    if ((s->ninact | s->nact | s->nsec) & 1) throw Error{DCG_E_ARG, "space sizes must be even (Kramers pairs)"};
    if (s->nsymrpa < 1 || !s->multb || !s->irpamo || !s->h_re || !s->h_im)
        throw Error{DCG_E_ARG, "missing symmetry tables or one-electron integrals"};
    if (s->nrec < 0 || (s->nrec > 0 && (!s->rec_ijkl || !s->rec_re))) throw Error{DCG_E_ARG, "missing records"};
    if (!s->realonly && s->nrec > 0 && !s->rec_im) throw Error{DCG_E_ARG, "complex system without rec_im"};
    c.ni = s->ninact; c.na = s->nact; c.ns = s->nsec; c.ne = s->nelec; c.nmo = s->nmo;
    c.nsym = s->nsymrpa; c.totsym = s->totsym; c.selectroot = s->selectroot; c.realonly = s->realonly != 0;
    c.eshift = s->eshift; c.ecore = s->ecore;
    c.ras1 = s->ras1_size; c.ras2 = s->ras2_size; c.ras3 = s->ras3_size;
    c.ras1_max_hole = s->ras1_max_hole; c.ras3_max_elec = s->ras3_max_elec;
    c.min_hole_ras1 = s->min_hole_ras1; c.min_elec_ras3 = s->min_elec_ras3;
    if (c.selectroot < 1) throw Error{DCG_E_ARG, "selectroot must be >= 1"};
    const int n = c.nsym, n2 = 2 * n;
    c.multb.assign(s->multb, s->multb + n2 * n2);
    c.irpamo.assign(s->irpamo, s->irpamo + c.nmo);
    for (int x : c.irpamo)
        if (x < 1 || x > n2) throw Error{DCG_E_ARG, "irpamo out of range"};
    // MULTB(i0, j0) column-major -> tables (read_mrconee.F90:368-453), stored [a-1][b-1]
    auto MB = [&](int i0, int j0) { return c.multb[(i0 - 1) + n2 * (j0 - 1)]; };
    std::vector<int> m2(n2 * n2, 0);
    for (int i0 = 1; i0 <= n2; i0++)
        for (int j0 = 1; j0 <= n2; j0++) {
            const int k0 = MB(i0, j0);
            if (k0 < 1 || k0 > n2) throw Error{DCG_E_ARG, "MULTB entry out of range"};
            m2[(i0 - 1) * n2 + (k0 - 1)] = j0;
        }
    c.multb_s.assign(n * n, 0);
    c.multb_d.assign(n * n, 0);
    c.multb_ds.assign(n * n, 0);
    for (int a = 1; a <= n; a++)
        for (int b = 1; b <= n; b++) {
            c.multb_s[(a - 1) * n + (b - 1)] = MB(a + n, b + n) - n;
            c.multb_d[(a - 1) * n + (b - 1)] = m2[(a - 1) * n2 + (b - 1)] - n;
            c.multb_ds[(a - 1) * n + (b - 1)] = MB(b + n, a);   // transpose(MULTB(n+1:2n, 1:n))
        }
    c.h.resize((size_t)c.nmo * c.nmo);
    for (size_t q = 0; q < c.h.size(); q++) c.h[q] = mk(s->h_re[q], s->h_im[q]);
    c.nrec = s->nrec;

    DevSystem &d = dev(c);
    d.h = upload(c, "sys.h", c.h);
    d.irp = upload(c, "sys.irp", c.irpamo);
    d.md = upload(c, "sys.md", c.multb_d);
    d.msy = upload(c, "sys.ms", c.multb_s);
    // integral expansion
    stage_begin(c, ST_INTS);
    const int nmoc = c.ni + c.na;
    const size_t ntw = (size_t)nmoc * nmoc * nmoc * nmoc;
    d.inttw = wsget<cplx>(c, "sys.inttw", ntw);
    DCG_CUDA(cudaMemsetAsync(d.inttw, 0, ntw * sizeof(cplx), c.stream));
    class_layout(c, d.cls);
    for (int id = 0; id < CL_COUNT; id++) {
        d.cls[id].p = wsget<cplx>(c, "sys.cls" + std::to_string(id), (size_t)d.cls[id].size);
        if (d.cls[id].size)
            DCG_CUDA(cudaMemsetAsync(d.cls[id].p, 0, (size_t)d.cls[id].size * sizeof(cplx), c.stream));
    }
    if (c.nrec > 0) {
        const int32_t *ijkl = s->rec_ijkl;
        const double *re = s->rec_re, *im = c.realonly ? nullptr : s->rec_im;
        if (!s->rec_on_device) {
            int32_t *dijkl = wsget<int32_t>(c, "rec.ijkl", (size_t)4 * c.nrec);
            double *dre = wsget<double>(c, "rec.re", (size_t)c.nrec);
            DCG_CUDA(cudaMemcpyAsync(dijkl, s->rec_ijkl, sizeof(int32_t) * 4 * c.nrec, cudaMemcpyHostToDevice, c.stream));
            DCG_CUDA(cudaMemcpyAsync(dre, s->rec_re, sizeof(double) * c.nrec, cudaMemcpyHostToDevice, c.stream));
            ijkl = dijkl;
            re = dre;
            if (im) {
                double *dim = wsget<double>(c, "rec.im", (size_t)c.nrec);
                DCG_CUDA(cudaMemcpyAsync(dim, s->rec_im, sizeof(double) * c.nrec, cudaMemcpyHostToDevice, c.stream));
                im = dim;
            }
        }
        size_t cls_bytes = 0;
        for (int id = 0; id < CL_COUNT; id++) cls_bytes += (size_t)d.cls[id].size * sizeof(cplx);
        FamScope fs(c, DCG_FAM_SCATTER, (double)c.nrec * (16.0 + (im ? 16.0 : 8.0)) + (double)cls_bytes + (double)ntw * sizeof(cplx));
        cplx *val = wsget<cplx>(c, "rec.val", (size_t)c.nrec);
        pack_cplx_kernel<<<grid1d(c.nrec, 256), 256, 0, c.stream>>>(re, im, c.nrec, val);
        DCG_LAUNCHED(c);
        launch_scatter(c, ijkl, val, c.nrec, d.inttw, d.cls);
    }
    stage_end(c, ST_INTS);
    fam_collect(c);
    c.have_system = true;
    c.have_casci = false;
}

// ------------------------------------------------------------------------- CASCI
// The dense eigensolver below kDavidsonMinDet determinants or for many roots; block Davidson
// on the resident Hamiltonian above it.
constexpr int kDavidsonMinDet = 600;
constexpr int kDavidsonMaxRoots = 12;

static bool use_davidson(const Context &c, int ndet, int nvec) {
    if (c.casci_solver == DCG_CASCI_DENSE) return false;
    const bool fits = nvec <= kDavidsonMaxRoots && ndet >= nvec + 5;
    if (c.casci_solver == DCG_CASCI_DAVIDSON) return fits;
    return fits && ndet >= kDavidsonMinDet;
}

// ------------------------------------------------------------------------- IVO
// r4divo.F90:80-93 / fockivo.F90:44-215 on the resident integrals: the number of HOMO spinors
// (fockivo.F90:49-53), the blocks of one abelian irrep of each Kramers pair per fermion-irrep
// group, and their eigenpairs (dcg_ivo.cu).
static void ivo(Context &c, int nfsym, const double *mo_energy, int nhomo, double *eps, double *u_re, double *u_im,
                int32_t *block_isym, int32_t *numh_out) {
    if (!c.have_system) throw Error{DCG_E_STATE, "dcg_ivo before dcg_set_system"};
    if (nfsym != 1 && nfsym != 2) throw Error{DCG_E_ARG, "IVO: nfsym must be 1 or 2"};
    if (!mo_energy || nhomo < 0) throw Error{DCG_E_ARG, "IVO: mo_energy missing or nhomo negative"};
    const int ni = c.ni, na = c.na, ns = c.ns, act_end = ni + na;
    int numh = nhomo;
    if (numh == 0) {
        if (c.ne + ni < 1) throw Error{DCG_E_ARG, "IVO: no occupied spinor"};
        const double eh = mo_energy[c.ne + ni - 1];
        for (int p = 0; p < act_end; p++)
            if (std::fabs(mo_energy[p] - eh) < 1.0e-1) numh++;
    }
    if (numh < 1 || numh > na) throw Error{DCG_E_ARG, "IVO: the HOMO spinors must lie in the active space"};
    std::vector<std::vector<int>> blocks;
    std::vector<int> bsym;
    for (int g = 0; g < nfsym; g++) {
        const int s0 = g == 0 ? 1 : c.nsym / 2 + 1, s1 = g == 0 ? c.nsym / 2 : c.nsym;
        for (int isym = s0; isym <= s1; isym += 2) {
            std::vector<int> L;
            for (int a = 0; a < ns; a++)
                if (c.irpamo[act_end + a] == isym) L.push_back(a);
            if (!L.empty()) {
                blocks.push_back(L);
                bsym.push_back(isym);
            }
        }
    }
    DevSystem &d = dev(c);
    std::vector<std::vector<double>> w;
    std::vector<std::vector<cplx>> v;
    ivo_blocks_eig(c, d.cls[CL_F1A].p, d.cls[CL_F2A].p, mo_energy + act_end, na - numh, na, c.ne % 2, (double)numh,
                   blocks, w, v);
    if (eps) std::fill(eps, eps + ns, 0.0);
    if (block_isym) std::fill(block_isym, block_isym + ns, 0);
    if (u_re) std::fill(u_re, u_re + (size_t)ns * ns, 0.0);
    if (u_im) std::fill(u_im, u_im + (size_t)ns * ns, 0.0);
    for (size_t b = 0; b < blocks.size(); b++) {
        const std::vector<int> &L = blocks[b];
        const size_t n = L.size();
        for (size_t i = 0; i < n; i++) {
            if (eps) eps[L[i]] = w[b][i];
            if (block_isym) block_isym[L[i]] = bsym[b];
            for (size_t j = 0; j < n; j++) {
                const cplx x = v[b][i + n * j];
                if (u_re) u_re[L[i] + (size_t)ns * L[j]] = x.x;
                if (u_im) u_im[L[i] + (size_t)ns * L[j]] = x.y;
            }
        }
    }
    if (numh_out) *numh_out = numh;
}

static int casci(Context &c, int nroot, double *eigen_out, double *ci_re, double *ci_im, int32_t *ndet_out) {
    if (!c.have_system) throw Error{DCG_E_STATE, "dcg_casci before dcg_set_system"};
    DevSystem &d = dev(c);
    c.dets = enumerate_ci(c);
    const int ndet = (int)c.dets.size();
    if (ndet_out) *ndet_out = ndet;
    if (ndet == 0) throw Error{DCG_E_NODET, "no CASCI configuration for totsym " + std::to_string(c.totsym)};
    if (c.selectroot > ndet) throw Error{DCG_E_ARG, "selectroot exceeds the number of CASCI configurations"};
    d.ndet = ndet;
    d.dets = upload(c, "ci.dets", c.dets);
    const int nr = std::max(1, std::min(nroot, ndet));
    const int nvec = std::max(nr, c.selectroot);
    double *w = wsget<double>(c, "ci.w", ndet);
    cplx *Z = wsget<cplx>(c, "ci.Z", (size_t)ndet * nvec);
    c.casci_iters = 0;
    if (use_davidson(c, ndet, nvec)) {
        // the Hamiltonian as CSR (singles and doubles of each determinant), never dense
        stage_begin(c, ST_CASMAT);
        CsrMatrix Hs;
        build_casmat_csr(c, d.dets, ndet, d.h, d.inttw, Hs);
        stage_end(c, ST_CASMAT);
        stage_begin(c, ST_CASEIG);
        // |r| <= 1e-13 max(1, max |H_ii|): eigenvalue errors ~|r|^2/gap, vector errors ~|r|/gap
        davidson_lowest_csr(c, Hs, nvec, w, Z, 1e-13, 400);
    } else {
        stage_begin(c, ST_CASMAT);
        cplx *H = wsget<cplx>(c, "ci.H", (size_t)ndet * ndet);
        launch_casmat(c, d.dets, ndet, d.h, d.inttw, H);
        stage_end(c, ST_CASMAT);
        stage_begin(c, ST_CASEIG);
        heev(c, ndet, H, ndet, w, 0, nvec, Z, ndet);
    }
    stage_end(c, ST_CASEIG);
    std::vector<double> wh = download(c, w, ndet);
    c.ecas.assign(wh.begin(), wh.begin() + nvec);
    for (double &x : c.ecas) x += c.ecore;   // casci.F90:72
    c.nroot_done = nvec;
    if (eigen_out)
        for (int r = 0; r < nr; r++) eigen_out[r] = c.ecas[r];
    d.c0 = wsget<cplx>(c, "ci.c0", ndet);
    DCG_CUDA(cudaMemcpyAsync(d.c0, Z + (size_t)ndet * (c.selectroot - 1), sizeof(cplx) * ndet,
                             cudaMemcpyDeviceToDevice, c.stream));
    if (ci_re) {
        std::vector<cplx> zh = download(c, Z, (size_t)ndet * nr);
        for (size_t q = 0; q < zh.size(); q++) {
            ci_re[q] = zh[q].x;
            if (ci_im) ci_im[q] = zh[q].y;
        }
    }
    DCG_CUDA(cudaStreamSynchronize(c.stream));
    c.have_casci = true;
    return 0;
}

// ------------------------------------------------------------------------- 4-index transformation
// (i'j'|k'l') = sum conj(U_ii') U_jj' conj(U_kk') U_ll' (ij|kl)   (module_intra.F90:130-277),
// index l first, then k, j, i, as four GEMMs.
// Quarters whose contracted orbital dimension exceeds this run on the split-precision tensor
// cores when the context asks for DCG_PREC_SPLIT.  Even a quarter over 12 or 20 orbitals is
// FP64-bound on a GB300 (8 M K^2 flops at ~1.2 TF/s against one pass over the class), so
// only trivial dimensions stay on the FP64 kernels.
constexpr int kSplitMinK = 4;

static void transform4(Context &c, const cplx *in, cplx *out, cplx *tmp, const int dm[4], const cplx *U[4]) {
    const int64_t d0 = dm[0], d1 = dm[1], d2 = dm[2], d3 = dm[3];
    const int64_t tot = d0 * d1 * d2 * d3;
    if (tot == 0) return;
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
    const bool split = c.precision == DCG_PREC_SPLIT;
    const int lb = c.split_lbo, sb = c.split_sbo;
    // l: tmp = in * U4
    if (split && d3 > kSplitMinK)
        zgemm_split(c, (int)(d0 * d1 * d2), (int)d3, (int)d3, 1, in, 1, d0 * d1 * d2, 0, U[3], d3, 0, tmp, 1,
                    d0 * d1 * d2, 0, false, lb, sb);
    else
        zgemm(c, OP_N, OP_N, (int)(d0 * d1 * d2), (int)d3, (int)d3, one, in, d0 * d1 * d2, 0, U[3], d3, 0, zero, tmp,
              d0 * d1 * d2, 0, 1);
    // k: out_l = tmp_l * conj(U3)
    if (split && d2 > kSplitMinK)
        zgemm_split(c, (int)(d0 * d1), (int)d2, (int)d2, (int)d3, tmp, 1, d0 * d1, d0 * d1 * d2, U[2], d2, 1, out, 1,
                    d0 * d1, d0 * d1 * d2, false, lb, sb);
    else
        zgemm(c, OP_N, OP_R, (int)(d0 * d1), (int)d2, (int)d2, one, tmp, d0 * d1, d0 * d1 * d2, U[2], d2, 0, zero,
              out, d0 * d1, d0 * d1 * d2, (int)d3);
    // j: tmp_kl = out_kl * U2
    if (split && d1 > kSplitMinK)
        zgemm_split(c, (int)d0, (int)d1, (int)d1, (int)(d2 * d3), out, 1, d0, d0 * d1, U[1], d1, 0, tmp, 1, d0,
                    d0 * d1, false, lb, sb);
    else
        zgemm(c, OP_N, OP_N, (int)d0, (int)d1, (int)d1, one, out, d0, d0 * d1, U[1], d1, 0, zero, tmp, d0, d0 * d1,
              (int)(d2 * d3));
    // i: out = U1^H * tmp, as out^T = tmp^T conj(U1) on the split path
    if (split && d0 > kSplitMinK)
        zgemm_split(c, (int)(d1 * d2 * d3), (int)d0, (int)d0, 1, tmp, d0, 1, 0, U[0], d0, 1, out, d0, 1, 0, false, lb,
                    sb);
    else
        zgemm(c, OP_C, OP_N, (int)d0, (int)(d1 * d2 * d3), (int)d0, one, U[0], d0, 0, tmp, d0, 0, zero, out, d0, 0,
              1);
}

// ------------------------------------------------------------------------- subspace block solve
// One symmetry block's share of the per-irrep results: solve_X_subspace prints e2X(isym) for a
// block whose S keeps dimm > 0 vectors above the cutoff (solve_A_subspace.F90:158-164,262).
static void sym_record(Context &c, int sub, int isym, double e2, double sc2, int dimm) {
    if (dimm <= 0) return;
    const size_t k = (size_t)sub * c.nsym + (size_t)(isym - 1);
    c.sym_e2[k] += e2;
    c.sym_sc2[k] += sc2;
    c.sym_printed[k] = 1;
}

// Vectors S keeps above the 1e-8 cutoff (cutoff.F90:37-70); S (dimn x dimn, upper triangle
// read) is destroyed.  Only for blocks without an outer index, where the count alone decides
// whether the reference prints a zero e2X(isym).
static int kept_count(Context &c, int dimn, cplx *S, int64_t lds) {
    double *w = wsget<double>(c, "blk.wcount", dimn);
    heev(c, dimn, S, lds, w, dimn, dimn, nullptr, dimn);   // values only
    const std::vector<double> wh = download(c, w, dimn);
    int kept = 0;
    for (double x : wh) kept += x >= 1.0e-8 ? 1 : 0;
    return kept;
}

struct BlockOut {
    double e2 = 0.0, sc2 = 0.0;
    int dimm = 0;
};

// Whether the E2 terms of a B' block come from its tridiagonal form (tridiag_e2) rather than
// its eigendecomposition: up to kTridiagE2MaxN, and when the outer index is not much longer
// than B' (the per-outer-index solves stream 5 words per element of VC through scratch; the
// eigenvector route reads VC once after one GEMM).
static bool tridiag_e2_pays(int dimm, int nouter) { return dimm <= kTridiagE2MaxN && nouter <= 2 * dimm; }

// Per outer index o: e2o = -sum_m |(W^H VC)_m,o|^2 / (alpha_o + w_m) and sco = sum_m
// |(W^H VC)_m,o|^2 / (alpha_o + w_m)^2 over the eigenpairs (w, W) of B' (dimm x dimm, destroyed;
// VC: dimm x nouter), as the reference's solve_X_subspace evaluates them.
static void e2_from_bprime(Context &c, int dimm, cplx *Bp, const cplx *VC, int nouter, const double *alpha,
                           double *e2o, double *sco) {
    if (tridiag_e2_pays(dimm, nouter) && band_e2_pays(dimm, nouter)) {   // band form, banded solves
        band_e2(c, 0, dimm, Bp, dimm, VC, dimm, nouter, alpha, e2o, sco);
        return;
    }
    if (tridiag_e2_pays(dimm, nouter)) {
        EigJob e;
        e.n = dimm;
        e.A = Bp;
        e.lda = dimm;
        e.slot = 0;
        e.tridiag_only = true;
        heev_values_batched(c, std::vector<EigJob>(1, e));
        tridiag_e2(c, 0, dimm, Bp, dimm, VC, dimm, nouter, alpha, e2o, sco);
        return;
    }
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
    double *wb = wsget<double>(c, "blk.wb", dimm);
    cplx *W = wsget<cplx>(c, "blk.W", (size_t)dimm * dimm);
    heev(c, dimm, Bp, dimm, wb, 0, dimm, W, dimm);
    cplx *VC1 = wsget<cplx>(c, "blk.VC1", (size_t)dimm * nouter);
    zgemm(c, OP_C, OP_N, dimm, nouter, dimm, one, W, dimm, 0, VC, dimm, 0, zero, VC1, dimm, 0, 1);
    launch_e2(c, VC1, dimm, nouter, alpha, wb, e2o, sco);
}

// The S-route products of B, D, E, F and G on the split path through the seven-slice kernel,
// by DCG_SROUTE_SPLIT_ACC (bit mask: 1 the B' build X^H (B X), 2 X^H Vsel, 4 the combined
// basis X W and (X W)^H Vsel; default 7, all three); FP64 otherwise.  On 20 inactive, 12
// active, 300 secondary spinors all three move no subspace E2 by more than 4e-13 Eh against
// the FP64 products and take the B-G stage from 20.9 to 14.7 ms.
static bool sroute_acc_split(const Context &c, int which) {
    if (c.precision != DCG_PREC_SPLIT) return false;
    static const int mask = [] {
        const char *e = getenv("DCG_SROUTE_SPLIT_ACC");
        return e ? atoi(e) : 7;
    }();
    return (mask & which) != 0;
}
// C (M x N, ld ldc) = A (M x K, ld lda) B (K x N, ld ldb)
static void prod_nn(Context &c, bool split, int M, int N, int K, const cplx *A, int64_t lda, const cplx *B,
                    int64_t ldb, cplx *C, int64_t ldc) {
    if (split) {
        zgemm_split_acc(c, M, N, K, 1, A, 1, lda, 0, B, ldb, 0, C, 1, ldc, 0, false);
    } else {
        const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
        zgemm(c, OP_N, OP_N, M, N, K, one, A, lda, 0, B, ldb, 0, zero, C, ldc, 0, 1);
    }
}
// C (M x N, ld ldc) = A^H B with A (K x M, ld lda), B (K x N, ld ldb); on the split path as
// its transpose B^T conj(A)
static void prod_cn(Context &c, bool split, int M, int N, int K, const cplx *A, int64_t lda, const cplx *B,
                    int64_t ldb, cplx *C, int64_t ldc) {
    if (split) {
        zgemm_split_acc(c, N, M, K, 1, B, ldb, 1, 0, A, lda, 1, C, ldc, 1, 0, false);
    } else {
        const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
        zgemm(c, OP_C, OP_N, M, N, K, one, A, lda, 0, B, ldb, 0, zero, C, ldc, 0, 1);
    }
}

// S,B (dimn x dimn) already assembled; Vsel (dimn x nouter); alphas on device.
static BlockOut solve_block(Context &c, int dimn, cplx *S, cplx *B, const cplx *Vsel, int nouter, const double *alpha) {
    BlockOut r;
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
    double *ws = wsget<double>(c, "blk.ws", dimn);
    // S eigenvalues first (cutoff count), then the kept eigenvectors
    std::vector<double> wsh;
    {
        double *dummy_w = ws;
        heev(c, dimn, S, dimn, dummy_w, dimn, dimn, nullptr, dimn);   // values only
        wsh = download(c, ws, dimn);
    }
    int vlo = dimn;
    for (int j = 0; j < dimn; j++)
        if (wsh[j] >= 1.0e-8) { vlo = j; break; }   // cutoff.F90:37-70 (ascending eigenvalues)
    const int dimm = dimn - vlo;
    r.dimm = dimm;
    if (dimm == 0 || nouter == 0) return r;
    // eigenvectors: re-run the vector stage on the still-reduced S (reflectors kept in S)
    cplx *X = wsget<cplx>(c, "blk.X", (size_t)dimn * dimm);
    heev_vectors_only(c, dimn, S, dimn, ws, vlo, dimn, X, dimn);
    launch_scale_cols(c, X, dimn, dimn, dimm, ws, vlo);   // X = U lambda^-1/2
    // B' = X^H B X
    cplx *BX = wsget<cplx>(c, "blk.BX", (size_t)dimn * dimm);
    cplx *Bp = wsget<cplx>(c, "blk.Bp", (size_t)dimm * dimm);
    prod_nn(c, sroute_acc_split(c, 1), dimn, dimm, dimn, B, dimn, X, dimn, BX, dimn);
    prod_cn(c, sroute_acc_split(c, 1), dimm, dimm, dimn, X, dimn, BX, dimn, Bp, dimm);
    herm_from_upper(c, dimm, Bp, dimm);
    double *e2o = wsget<double>(c, "blk.e2o", nouter);
    double *sco = wsget<double>(c, "blk.sco", nouter);
    cplx *VC0 = wsget<cplx>(c, "blk.VC0", (size_t)dimm * nouter);
    if (tridiag_e2_pays(dimm, nouter)) {
        prod_cn(c, sroute_acc_split(c, 2), dimm, nouter, dimn, X, dimn, Vsel, dimn, VC0, dimm);
        e2_from_bprime(c, dimm, Bp, VC0, nouter, alpha, e2o, sco);
    } else {
        // B' = W w W^H, then the outer-index vectors in the combined basis (X W)^H Vsel: one
        // product over the long outer index instead of X^H Vsel followed by W^H (X^H Vsel)
        double *wb = wsget<double>(c, "blk.wb", dimm);
        cplx *W = wsget<cplx>(c, "blk.W", (size_t)dimm * dimm);
        heev(c, dimm, Bp, dimm, wb, 0, dimm, W, dimm);
        cplx *XW = wsget<cplx>(c, "blk.XW", (size_t)dimn * dimm);
        prod_nn(c, sroute_acc_split(c, 4), dimn, dimm, dimm, X, dimn, W, dimm, XW, dimn);
        prod_cn(c, sroute_acc_split(c, 4), dimm, nouter, dimn, XW, dimn, Vsel, dimn, VC0, dimm);
        launch_e2(c, VC0, dimm, nouter, alpha, wb, e2o, sco);
    }
    double *red = wsget<double>(c, "blk.red", 2);
    dsum(c, e2o, nouter, red);
    dsum(c, sco, nouter, red + 1);
    std::vector<double> hr = download(c, red, 2);
    r.e2 = hr[0];
    r.sc2 = hr[1];
    return r;
}

// A block of B, D, E, F or G queued for the joint solve: its S, B and outer-index vectors
// in buffers of its own (named per job), so the blocks of every subspace can be reduced
// together once all are built.
struct BlockJob {
    int sub;          // subspace index, 0 A .. 7 H
    int isym;         // symmetry block
    int dimn, nouter;
    cplx *S, *B, *Vsel;
    double *alpha;
};

// solve_block for many blocks at once: their S matrices reduced in shared batched launches
// (at most kEigSlots at a time), the cutoff and B' per block, then their B' matrices reduced
// together the same way; the per-block E2 as solve_block forms it.  The tridiagonal loops of
// independent blocks overlap instead of adding.
static void solve_block_jobs(Context &c, std::vector<BlockJob> &all, double e2_sub[8], double sc2_sub[8]) {
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
    auto nm = [](const char *b, size_t j) { return std::string(b) + "#" + std::to_string(j); };
    for (size_t p0 = 0; p0 < all.size(); p0 += kEigSlots) {
        const size_t np = std::min<size_t>(kEigSlots, all.size() - p0);
        std::vector<double *> ws(np), wb(np, nullptr), red(np);
        std::vector<cplx *> X(np, nullptr), Bp(np, nullptr);
        std::vector<int> dimm(np, 0);
        std::vector<bool> band(np, false);
        // S: eigenvalues together, then each block's cutoff, kept vectors and B'
        std::vector<EigJob> es;
        for (size_t j = 0; j < np; j++) {
            BlockJob &b = all[p0 + j];
            ws[j] = wsget<double>(c, nm("bj.ws", j), b.dimn);
            EigJob e;
            e.n = b.dimn;
            e.A = b.S;
            e.lda = b.dimn;
            e.w = ws[j];
            e.slot = (int)j;
            es.push_back(e);
        }
        heev_values_batched(c, es);
        std::vector<std::vector<double>> wsh(np);
        for (size_t j = 0; j < np; j++) {
            wsh[j].resize(all[p0 + j].dimn);
            DCG_CUDA(cudaMemcpyAsync(wsh[j].data(), ws[j], sizeof(double) * wsh[j].size(), cudaMemcpyDeviceToHost,
                                     c.stream));
        }
        DCG_CUDA(cudaStreamSynchronize(c.stream));
        std::vector<int> vlo(np, 0);
        std::vector<VecJob> xv;
        for (size_t j = 0; j < np; j++) {
            BlockJob &b = all[p0 + j];
            vlo[j] = b.dimn;
            for (int q = 0; q < b.dimn; q++)
                if (wsh[j][q] >= 1.0e-8) {   // cutoff.F90:37-70 (ascending eigenvalues)
                    vlo[j] = q;
                    break;
                }
            dimm[j] = b.dimn - vlo[j];
            if (dimm[j] == 0 || b.nouter == 0) continue;
            X[j] = wsget<cplx>(c, nm("bj.X", j), (size_t)b.dimn * dimm[j]);
            VecJob v;
            v.slot = (int)j;
            v.n = v.lda = v.ldz = b.dimn;
            v.A = b.S;
            v.vlo = vlo[j];
            v.vhi = b.dimn;
            v.Z = X[j];
            xv.push_back(v);
        }
        eig_slot_jobs(c, xv, {});   // the kept S eigenvectors of every block, overlapped
        std::vector<EigJob> eb;
        for (size_t j = 0; j < np; j++) {
            BlockJob &b = all[p0 + j];
            if (!X[j]) continue;
            launch_scale_cols(c, X[j], b.dimn, b.dimn, dimm[j], ws[j], vlo[j]);   // X = U lambda^-1/2
            cplx *BX = wsget<cplx>(c, "bj.BX", (size_t)b.dimn * dimm[j]);
            Bp[j] = wsget<cplx>(c, nm("bj.Bp", j), (size_t)dimm[j] * dimm[j]);
            prod_nn(c, sroute_acc_split(c, 1), b.dimn, dimm[j], b.dimn, b.B, b.dimn, X[j], b.dimn, BX, b.dimn);
            prod_cn(c, sroute_acc_split(c, 1), dimm[j], dimm[j], b.dimn, X[j], b.dimn, BX, b.dimn, Bp[j], dimm[j]);
            herm_from_upper(c, dimm[j], Bp[j], dimm[j]);
            wb[j] = wsget<double>(c, nm("bj.wb", j), dimm[j]);
            if (tridiag_e2_pays(dimm[j], b.nouter) && band_e2_pays(dimm[j], b.nouter)) {
                band[j] = true;   // E2 from its band form below, no tridiagonal reduction
                continue;
            }
            EigJob e;
            e.n = dimm[j];
            e.A = Bp[j];
            e.lda = dimm[j];
            e.w = wb[j];
            e.slot = (int)j;
            e.tridiag_only = tridiag_e2_pays(dimm[j], b.nouter);
            eb.push_back(e);
        }
        // B': reductions together, then E2 per block (tridiagonal form, or eigenvectors and
        // one product over the outer index in the combined basis X W)
        heev_values_batched(c, eb);
        std::vector<VecJob> wv;
        std::vector<TE2Job> tv;
        std::vector<cplx *> W(np, nullptr);
        std::vector<double *> e2o(np, nullptr), sco(np, nullptr);
        for (size_t j = 0; j < np; j++) {
            BlockJob &b = all[p0 + j];
            if (!Bp[j]) continue;
            const int m = dimm[j];
            e2o[j] = wsget<double>(c, nm("bj.e2o", j), b.nouter);
            sco[j] = wsget<double>(c, nm("bj.sco", j), b.nouter);
            if (band[j]) {
                cplx *VC = wsget<cplx>(c, nm("bj.VC", j), (size_t)m * b.nouter);
                prod_cn(c, sroute_acc_split(c, 2), m, b.nouter, b.dimn, X[j], b.dimn, b.Vsel, b.dimn, VC, m);
                band_e2(c, (int)j, m, Bp[j], m, VC, m, b.nouter, b.alpha, e2o[j], sco[j]);
            } else if (tridiag_e2_pays(m, b.nouter)) {
                cplx *VC = wsget<cplx>(c, nm("bj.VC", j), (size_t)m * b.nouter);
                prod_cn(c, sroute_acc_split(c, 2), m, b.nouter, b.dimn, X[j], b.dimn, b.Vsel, b.dimn, VC, m);
                TE2Job t;
                t.slot = (int)j;
                t.n = m;
                t.A = Bp[j];
                t.lda = t.ldvc = m;
                t.VC = VC;
                t.nouter = b.nouter;
                t.alpha = b.alpha;
                t.e2o = e2o[j];
                t.sco = sco[j];
                tv.push_back(t);
            } else {
                W[j] = wsget<cplx>(c, nm("bj.W", j), (size_t)m * m);
                VecJob v;
                v.slot = (int)j;
                v.n = v.lda = v.ldz = m;
                v.A = Bp[j];
                v.vlo = 0;
                v.vhi = m;
                v.Z = W[j];
                wv.push_back(v);
            }
        }
        eig_slot_jobs(c, wv, tv);   // B' of every block, overlapped
        for (size_t j = 0; j < np; j++) {
            BlockJob &b = all[p0 + j];
            if (!Bp[j]) continue;
            const int m = dimm[j];
            if (W[j]) {
                cplx *VC = wsget<cplx>(c, "bj.VCw", (size_t)m * b.nouter);
                cplx *XW = wsget<cplx>(c, "bj.XW", (size_t)b.dimn * m);
                prod_nn(c, sroute_acc_split(c, 4), b.dimn, m, m, X[j], b.dimn, W[j], m, XW, b.dimn);
                prod_cn(c, sroute_acc_split(c, 4), m, b.nouter, b.dimn, XW, b.dimn, b.Vsel, b.dimn, VC, m);
                launch_e2(c, VC, m, b.nouter, b.alpha, wb[j], e2o[j], sco[j]);
            }
            red[j] = wsget<double>(c, nm("bj.red", j), 2);
            dsum(c, e2o[j], b.nouter, red[j]);
            dsum(c, sco[j], b.nouter, red[j] + 1);
        }
        for (size_t j = 0; j < np; j++) {
            if (!Bp[j]) continue;
            const std::vector<double> hr = download(c, red[j], 2);
            e2_sub[all[p0 + j].sub] += hr[0];
            sc2_sub[all[p0 + j].sub] += hr[1];
            sym_record(c, all[p0 + j].sub, all[p0 + j].isym, hr[0], hr[1], dimm[j]);
        }
    }
}

}  // namespace dcg

namespace dcg {

// ------------------------------------------------------------------------- densities
// psi (full N-space) -> Ycat = [E_pq psi | E_pq psit] (M x 2na^2), Zcat = E_cd Ycat
// (M x na^2 x 2na^2) stored right after Ycat, then Gall = Ycat(:, :na^2)^H [Ycat | Zcat]
// and G1 = psi^H Ycat.  These are the reference's dim1..dim4_density values for every
// index combination at once (density_matrix.F90:3-247): <0|E_ab X|0> with
// <0|E_ab = (E_ba|0>)^H, and an unrestricted intermediate determinant space.
struct RdmBufs {
    cplx *g1 = nullptr, *gall = nullptr;
    const cplx *Y = nullptr;   // E_pq psi over the full space (M x na^2, column p + na q)
    int64_t M = 0;
    RDMView view;
};

static RdmBufs rdm_build(Context &c, const uint64_t *full, int64_t M, const cplx *psi, const double *eps_act,
                         bool third) {
    const int na = c.na;
    const int64_t na2 = (int64_t)na * na, na4 = na2 * na2;
    RdmBufs r;
    const int nv = eps_act ? 2 : 1;
    cplx *vin = wsget<cplx>(c, "rdm.vin", (size_t)M * nv);
    DCG_CUDA(cudaMemcpyAsync(vin, psi, sizeof(cplx) * M, cudaMemcpyDeviceToDevice, c.stream));
    if (eps_act) launch_occ_energy(c, na, M, full, eps_act, psi, vin + M);
    const int64_t ncol = nv * na2 + (third ? nv * na4 : 0);
    cplx *YZ = wsget<cplx>(c, "rdm.YZ", (size_t)M * ncol);
    launch_apply_E(c, na, M, full, vin, nv, YZ);
    if (third) launch_apply_E(c, na, M, full, YZ, (int)(nv * na2), YZ + M * nv * na2);
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
    FamScope fs(c, DCG_FAM_RDM, 8.0 * (double)M * (double)nv * na2 + 8.0 * (double)na2 * ncol * M);
    r.g1 = wsget<cplx>(c, "rdm.g1", (size_t)nv * na2);
    zgemm(c, OP_C, OP_N, 1, (int)(nv * na2), (int)M, one, psi, M, 0, YZ, M, 0, zero, r.g1, 1, 0, 1);
    r.gall = wsget<cplx>(c, "rdm.gall", (size_t)na2 * ncol);
    if (c.precision == DCG_PREC_SPLIT && M > 32 && ncol >= 128) {
        // gall^T = [Y|Z]^T conj(Y) on the split-precision tensor cores (rows of [Y|Z]^T are
        // its columns, contiguous along the determinant index)
        zgemm_split(c, (int)ncol, (int)na2, (int)M, 1, YZ, M, 1, 0, YZ, M, 1, r.gall, na2, 1, 0, false, c.split_lbo,
                    c.split_sbo);
    } else {
        zgemm(c, OP_C, OP_N, (int)na2, (int)ncol, (int)M, one, YZ, M, 0, YZ, M, 0, zero, r.gall, na2, 0, 1);
    }
    r.Y = YZ;
    r.M = M;
    r.view.na = na;
    r.view.g1 = r.g1;
    r.view.t1 = eps_act ? r.g1 + na2 : nullptr;
    r.view.g2 = r.gall;
    r.view.t2 = eps_act ? r.gall + na2 * na2 : nullptr;
    r.view.g3 = third ? r.gall + nv * na2 * na2 : nullptr;
    r.view.t3 = (third && eps_act) ? r.view.g3 + na4 * na2 : nullptr;
    return r;
}

// ------------------------------------------------------------------------- e0test
// e0test (e0test.F90:4-272), which r4dcasci runs after the CASCI (r4dcasci.F90:89): the
// HF-like energy of the lowest ninact + nelec spinors and the selected root's energy from its
// 1- and 2-RDM in four parts, against eigen - ecore.  The RDMs come from the device (the
// density GEMMs in FP64 whatever the context's precision); the na^4 and nmoc^2 sums run on
// the host.  out: energyHF(1), energyHF(2), energy 1..4, their sum, and eigen - ecore - sum.
static void e0test(Context &c, double *out) {
    if (!c.have_casci) throw Error{DCG_E_STATE, "dcg_casci_energy_check before dcg_casci"};
    DevSystem &d = dev(c);
    const int ni = c.ni, na = c.na, nmoc = ni + na, nmo = c.nmo;
    const std::vector<uint64_t> full = gosper_all(na, c.ne);
    const int64_t M = (int64_t)full.size();
    std::vector<int64_t> pos(d.ndet);
    for (int i = 0; i < d.ndet; i++) pos[i] = std::lower_bound(full.begin(), full.end(), c.dets[i]) - full.begin();
    uint64_t *d_full = upload(c, "e0.full", full);
    int64_t *d_pos = upload(c, "e0.pos", pos);
    cplx *psi = wsget<cplx>(c, "e0.psi", (size_t)M);
    launch_embed(c, d.ndet, d_pos, d.c0, psi, M);
    const int prec = c.precision;
    c.precision = DCG_PREC_FP64;
    RdmBufs r;
    try {
        r = rdm_build(c, d_full, M, psi, nullptr, false);
    } catch (...) {
        c.precision = prec;
        throw;
    }
    c.precision = prec;
    const size_t na2 = (size_t)na * na;
    const std::vector<cplx> g1 = download(c, r.g1, na2);                 // <E_pq> at p + na q
    const std::vector<cplx> gall = download(c, r.gall, na2 * na2);       // <E_qp E_rs> at (p + na q) + na^2 (r + na s)
    const std::vector<cplx> h = download(c, d.h, (size_t)nmo * nmo);
    const std::vector<cplx> g = download(c, d.inttw, (size_t)nmoc * nmoc * nmoc * nmoc);
    auto G = [&](int p, int q, int rr, int ss) {
        return g[p + (size_t)nmoc * (q + (size_t)nmoc * (rr + (size_t)nmoc * ss))];
    };
    auto D1 = [&](int i, int j) { return g1[i + (size_t)na * j]; };
    auto D2 = [&](int i, int j, int k, int l) { return gall[(j + (size_t)na * i) + na2 * (k + (size_t)na * l)]; };
    auto cs = [](cplx a, cplx b) { return cadd(a, b); };
    cplx hf1 = mk(0.0, 0.0), hf2 = mk(0.0, 0.0), e1 = mk(0.0, 0.0), e2 = mk(0.0, 0.0), e3 = mk(0.0, 0.0),
         e4 = mk(0.0, 0.0);
    const int nocc = ni + c.ne;
    for (int i = 0; i < nocc; i++) hf1 = cs(hf1, h[i + (size_t)nmo * i]);
    for (int i = 0; i < nocc; i++)
        for (int j = i; j < nocc; j++) hf2 = cs(hf2, csub(G(i, i, j, j), G(i, j, j, i)));
    hf2 = cscale(hf2, 0.5);
    hf2 = cadd(hf2, cconj(hf2));
    for (int i = 0; i < ni; i++) e1 = cs(e1, h[i + (size_t)nmo * i]);
    for (int i = 0; i < ni; i++)
        for (int j = i; j < ni; j++) e2 = cs(e2, csub(G(i, i, j, j), G(i, j, j, i)));
    e2 = cscale(e2, 0.5);
    e2 = cadd(e2, cconj(e2));
    for (int i = ni; i < nmoc; i++)
        for (int j = i; j < nmoc; j++) {
            cplx one = h[i + (size_t)nmo * j];
            for (int k = 0; k < ni; k++) one = cadd(one, csub(G(i, j, k, k), G(i, k, k, j)));
            if (i == j) one = cscale(one, 0.5);
            e3 = cadd(e3, cmul(one, D1(i - ni, j - ni)));
        }
    e3 = cadd(e3, cconj(e3));
    for (int i = 0; i < na; i++)
        for (int j = 0; j < na; j++)
            for (int k = 0; k < na; k++)
                for (int l = 0; l < na; l++) {
                    const cplx x = G(ni + i, ni + j, ni + k, ni + l);
                    e4 = cadd(e4, cmul(D2(i, j, k, l), x));
                    if (j == k) e4 = csub(e4, cmul(D1(i, l), x));
                }
    e4 = cscale(e4, 0.5);
    const double t = e1.x + e2.x + e3.x + e4.x;
    out[0] = hf1.x;
    out[1] = hf2.x;
    out[2] = e1.x;
    out[3] = e2.x;
    out[4] = e3.x;
    out[5] = e4.x;
    out[6] = t;
    out[7] = (c.ecas[c.selectroot - 1] - c.ecore) - t;
}

// ------------------------------------------------------------------------- subspace drivers
struct SubCtx {
    Context *c;
    RDMView rv;
    const double *eps_act_d;   // device, active orbital energies
    std::vector<double> eps;   // host, global
    double e0;
    const cplx *Y = nullptr;   // E_pq psi over the full nelec-electron space (M x na^2)
    int64_t M = 0;
    struct GramJob *defer = nullptr;   // when set, Gram-route blocks are queued here (see GramJob)
    std::vector<struct GramJob> *jobs = nullptr;
    std::vector<BlockJob> *bjobs = nullptr;   // when set, S/B-route blocks are queued here
};

struct BlockSpec {
    std::vector<int> ind;             // flattened tuples
    int dimn = 0;
    int isym = 1;                     // the symmetry block's isym (solve_X_subspace's loop index)
    std::vector<int64_t> outer_off;   // into V
    std::vector<int64_t> inner_off;   // into V
    std::vector<double> alpha;
};

// Subspace blocks A and C through the Gram factor of their overlap (S = G^H G, B = G^H D G,
// G of size Mp x dimn over the (nelec +- 1)-electron determinants).  With G = P Sigma Q^H,
// the kept eigenvectors of S are U = G^H P Lambda^-1/2 (Lambda = Sigma^2, the eigenvalues of
// K = G G^H, which are those of S), so that
//   X = U Lambda^-1/2 = G^H P Lambda^-1,   X^H v = Lambda^-1 P^H (G v),   B' = X^H B X = P^H D P.
// The reference's 1e-8 cutoff is applied to the eigenvalues of K.  E2 is invariant to the basis
// chosen inside the kept space, so this reproduces solve_block on (S, B) with an Mp x Mp
// eigenproblem instead of a dimn x dimn one.
// E2 terms of a Gram block whose metric K = G G^H keeps all its eigenvalues: with K = P L P^H
// unitary, X = G^H P L^-1, B' = P^H D P and Xv = L^-1 P^H G v, so
//   -v~^H (B' + a)^-1 v~ = -u^H (D + a)^-1 u,   |(B' + a)^-1 v~|^2 = |(D + a)^-1 u|^2,
// u = P v~ = K^-1 G v: one Cholesky solve with K instead of the eigendecompositions of K and
// B'.  K is destroyed (overwritten by its factor).  e2o, sco: device, nouter entries.
static void gram_cholesky_e2(Context &c, int Mp, int dimn, const cplx *G, cplx *K, const double *Dd,
                             const cplx *Vsel, int nouter, const double *alpha, int tag, const double *&e2o_out,
                             const double *&sco_out) {
    const std::string t = "#" + std::to_string(tag);
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
    int *info = wsget<int>(c, "gram.info2" + t, 1);
    zpotrf_lower(c, Mp, K, Mp, info);
    cplx *U = wsget<cplx>(c, "gram.U" + t, (size_t)Mp * nouter);
    zgemm(c, OP_N, OP_N, Mp, nouter, dimn, one, G, Mp, 0, Vsel, dimn, 0, zero, U, Mp, 0, 1);
    zpotrs_lower(c, Mp, K, Mp, U, Mp, nouter);
    double *e2o = wsget<double>(c, "gram.e2o" + t, nouter);
    double *sco = wsget<double>(c, "gram.sco" + t, nouter);
    launch_e2(c, U, Mp, nouter, alpha, Dd, e2o, sco);
    c.gram_cholesky_blocks++;
    e2o_out = e2o;
    sco_out = sco;
}

// Largest number of metric eigenvalues under the cutoff that the complement route takes.
// Up to this many, the deflated route costs less than the eigendecompositions of K and B': its
// packed-pair GEMM (r^2 Mp nouter / 2) and per-index r x r solves grow as r^2 and r^3 (at
// 12 active, 792 determinants, r = 162 made the A/C stage 2x slower than the eigen route).
constexpr int kWoodburyMaxR = 64;

// E2 terms of a Gram block whose metric K keeps all but its r smallest eigenpairs (Ps, Mp x r,
// the eigenvectors under the cutoff; lam_max its largest eigenvalue).  With P the kept
// eigenvectors, u = P v~ = sum_kept p lam^-1 p^H G v = K'^-1 (1 - Ps Ps^H) G v for
// K' = K + s Ps Ps^H (s = max(1, lam_max): K' keeps the kept eigenpairs and is well
// conditioned), and B' = P^H D P is the compression of D to the complement of Ps, whose
// inverse there gives e2 and c^2 per outer index (launch_woodbury_e2).  The reference's
// eigendecomposition of B' and the back-transformation of every kept vector are replaced by
// r vectors, one Cholesky solve and an r x r system per outer index.  Kc (a copy of K) is
// destroyed.
static void gram_woodbury_e2(Context &c, int Mp, int dimn, const cplx *G, cplx *Kc, const cplx *Ps, int r,
                             double lam_max, const double *Dd, const cplx *Vsel, int nouter, const double *alpha,
                             int tag, const double *&e2o_out, const double *&sco_out) {
    const std::string t = "#" + std::to_string(tag);
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0), mone = mk(-1.0, 0.0);
    const double sh = std::max(1.0, lam_max);
    zgemm(c, OP_N, OP_C, Mp, Mp, r, mk(sh, 0.0), Ps, Mp, 0, Ps, Mp, 0, one, Kc, Mp, 0, 1);   // K' = K + s Ps Ps^H
    int *info = wsget<int>(c, "gram.winfo" + t, 1);
    zpotrf_lower(c, Mp, Kc, Mp, info);
    cplx *U = wsget<cplx>(c, "gram.U" + t, (size_t)Mp * nouter);
    zgemm(c, OP_N, OP_N, Mp, nouter, dimn, one, G, Mp, 0, Vsel, dimn, 0, zero, U, Mp, 0, 1);
    cplx *Q = wsget<cplx>(c, "gram.Q" + t, (size_t)r * nouter);
    zgemm(c, OP_C, OP_N, r, nouter, Mp, one, Ps, Mp, 0, U, Mp, 0, zero, Q, r, 0, 1);
    zgemm(c, OP_N, OP_N, Mp, nouter, r, mone, Ps, Mp, 0, Q, r, 0, one, U, Mp, 0, 1);   // (1 - Ps Ps^H) G v
    zpotrs_lower(c, Mp, Kc, Mp, U, Mp, nouter);
    double *e2o = wsget<double>(c, "gram.e2o" + t, nouter);
    double *sco = wsget<double>(c, "gram.sco" + t, nouter);
    launch_woodbury_e2(c, Mp, r, U, Mp, Ps, Mp, Dd, alpha, nouter, e2o, sco);
    int h = 0;
    DCG_CUDA(cudaMemcpyAsync(&h, info, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    DCG_CUDA(cudaStreamSynchronize(c.stream));
    if (h != 0) throw Error{DCG_E_NUMERIC, "deflated Gram metric is not positive definite"};
    c.gram_woodbury_blocks++;
    e2o_out = e2o;
    sco_out = sco;
}

// B' = P^H (D P) (dm x dm) from P and PD (Mp x dm).  Unlike the metric K and Lambda^-1 P^H G v,
// B' is not amplified by Lambda^-1 (P is orthonormal and D diagonal), so on the split path it
// runs on the tensor cores, as its transpose (D P)^T conj(P) written back transposed.
static void bprime_product(Context &c, int Mp, int dm, const cplx *P, const cplx *PD, cplx *Bp) {
    if (c.precision == DCG_PREC_SPLIT && dm > kSplitMinK) {
        zgemm_split(c, dm, dm, Mp, 1, PD, Mp, 1, 0, P, Mp, 1, Bp, dm, 1, 0, false, c.split_lbo, c.split_sbo);
    } else {
        const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
        zgemm(c, OP_C, OP_N, dm, dm, Mp, one, P, Mp, 0, PD, Mp, 0, zero, Bp, dm, 0, 1);
    }
}

// The Gram-route products whose errors Lambda^-1 amplifies: the metric K = G G^H, G v and
// P^H (G v).  On the split path the first two run on the tensor cores through the seven-slice
// product (~2^-45 of row max x column max per term; the five-slice product moved e2c by 1.2e-9 Eh
// on 20/12/300 when it carried K).  Measured there against the oracle, K and G v on seven slices
// change no e2 by more than 3e-12 Eh; P^H (G v) on seven slices moved e2c by 2.2e-10 Eh (its
// outputs along the modes near the cutoff are ~1e-4 of its inputs and are divided by Lambda next),
// so it stays in FP64.  which: 1 the metric, 2 G v, 4 P^H (G v); DCG_GRAM_SPLIT_ACC is a mask of
// them (default 3; 0 keeps all three in FP64).
static bool gram_acc_split(const Context &c, int which) {
    if (c.precision != DCG_PREC_SPLIT) return false;
    const char *e = getenv("DCG_GRAM_SPLIT_ACC");
    const int mask = e ? atoi(e) : 3;
    return (mask & which) != 0;
}
// K = G G^H (Mp x Mp; at least the upper triangle, the caller mirrors it)
static void gram_metric(Context &c, int Mp, int dimn, const cplx *G, cplx *K) {
    if (gram_acc_split(c, 1)) zgemm_split_acc(c, Mp, Mp, dimn, 1, G, 1, Mp, 0, G, Mp, 3, K, 1, Mp, 0, false);
    else zherk_upper(c, Mp, dimn, G, Mp, K, Mp);
}
// GV = G Vsel (Mp x nouter)
static void gram_gv(Context &c, int Mp, int nouter, int dimn, const cplx *G, const cplx *Vsel, cplx *GV) {
    if (gram_acc_split(c, 2)) {
        zgemm_split_acc(c, Mp, nouter, dimn, 1, G, 1, Mp, 0, Vsel, dimn, 0, GV, 1, Mp, 0, false);
    } else {
        const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
        zgemm(c, OP_N, OP_N, Mp, nouter, dimn, one, G, Mp, 0, Vsel, dimn, 0, zero, GV, Mp, 0, 1);
    }
}
// VC0 = P^H GV (dm x nouter), on the split path as its transpose GV^T conj(P)
static void gram_phgv(Context &c, int dm, int nouter, int Mp, const cplx *P, const cplx *GV, cplx *VC0) {
    if (gram_acc_split(c, 4)) {
        zgemm_split_acc(c, nouter, dm, Mp, 1, GV, Mp, 1, 0, P, Mp, 1, VC0, dm, 1, 0, false);
    } else {
        const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
        zgemm(c, OP_C, OP_N, dm, nouter, Mp, one, P, Mp, 0, GV, Mp, 0, zero, VC0, dm, 0, 1);
    }
}

static BlockOut solve_gram_block(Context &c, int Mp, int dimn, const cplx *G, const double *Dd, const cplx *Vsel,
                                 int nouter, const double *alpha) {
    BlockOut r;
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
    // K is the overlap metric itself: its small eigenvalues (down to the 1e-8 cutoff) set X through
    // Lambda^-1, and an error in K moves their eigenvectors by |dK| / gap (see gram_metric).
    cplx *K = wsget<cplx>(c, "gram.K", (size_t)Mp * Mp);
    gram_metric(c, Mp, dimn, G, K);
    herm_from_upper(c, Mp, K, Mp);
    cplx *Kc = nullptr;
    if (c.metric_solver == DCG_METRIC_AUTO && nouter > 0) {   // kept for the Cholesky route
        Kc = wsget<cplx>(c, "gram.Kc", (size_t)Mp * Mp);
        DCG_CUDA(cudaMemcpyAsync(Kc, K, sizeof(cplx) * (size_t)Mp * Mp, cudaMemcpyDeviceToDevice, c.stream));
    }
    double *wk = wsget<double>(c, "gram.wk", Mp);
    heev(c, Mp, K, Mp, wk, Mp, Mp, nullptr, Mp);   // values first (cutoff count)
    std::vector<double> wh = download(c, wk, Mp);
    int vlo = Mp;
    for (int j = 0; j < Mp; j++)
        if (wh[j] >= 1.0e-8) { vlo = j; break; }   // cutoff.F90:37-70
    const int dimm = Mp - vlo;
    r.dimm = dimm;
    if (dimm == 0 || nouter == 0) return r;
    if (Kc && vlo <= kWoodburyMaxR) {   // Cholesky route (none under the cutoff) or its deflated form
        const double *e2o = nullptr, *sco = nullptr;
        if (vlo == 0) {
            gram_cholesky_e2(c, Mp, dimn, G, Kc, Dd, Vsel, nouter, alpha, 0, e2o, sco);
        } else {
            cplx *Ps = wsget<cplx>(c, "gram.Ps", (size_t)Mp * vlo);
            heev_vectors_only(c, Mp, K, Mp, wk, 0, vlo, Ps, Mp);
            gram_woodbury_e2(c, Mp, dimn, G, Kc, Ps, vlo, wh.back(), Dd, Vsel, nouter, alpha, 0, e2o, sco);
        }
        double *red = wsget<double>(c, "blk.red", 2);
        dsum(c, e2o, nouter, red);
        dsum(c, sco, nouter, red + 1);
        std::vector<double> hr = download(c, red, 2);
        r.e2 = hr[0];
        r.sc2 = hr[1];
        return r;
    }
    cplx *P = wsget<cplx>(c, "gram.P", (size_t)Mp * dimm);
    heev_vectors_only(c, Mp, K, Mp, wk, vlo, Mp, P, Mp);
    // VC0 = Lambda^-1 P^H (G v)
    cplx *GV = wsget<cplx>(c, "gram.GV", (size_t)Mp * nouter);
    gram_gv(c, Mp, nouter, dimn, G, Vsel, GV);
    cplx *VC0 = wsget<cplx>(c, "blk.VC0", (size_t)dimm * nouter);
    gram_phgv(c, dimm, nouter, Mp, P, GV, VC0);
    launch_scale_rows(c, dimm, nouter, VC0, dimm, wk, vlo, true);
    // B' = P^H D P
    cplx *PD = wsget<cplx>(c, "gram.PD", (size_t)Mp * dimm);
    DCG_CUDA(cudaMemcpyAsync(PD, P, sizeof(cplx) * (size_t)Mp * dimm, cudaMemcpyDeviceToDevice, c.stream));
    launch_scale_rows(c, Mp, dimm, PD, Mp, Dd, 0, false);
    cplx *Bp = wsget<cplx>(c, "blk.Bp", (size_t)dimm * dimm);
    bprime_product(c, Mp, dimm, P, PD, Bp);
    herm_from_upper(c, dimm, Bp, dimm);
    double *e2o = wsget<double>(c, "blk.e2o", nouter);
    double *sco = wsget<double>(c, "blk.sco", nouter);
    e2_from_bprime(c, dimm, Bp, VC0, nouter, alpha, e2o, sco);
    double *red = wsget<double>(c, "blk.red", 2);
    dsum(c, e2o, nouter, red);
    dsum(c, sco, nouter, red + 1);
    std::vector<double> hr = download(c, red, 2);
    r.e2 = hr[0];
    r.sc2 = hr[1];
    return r;
}

// A Gram-route block (subspace A or C) queued for the joint solve: the blocks of A and C are
// independent, so their K and B' eigenproblems are reduced together in batched launches.
struct GramJob {
    int Mp = 0, dimn = 0, nouter = 0;
    cplx *G = nullptr, *Vsel = nullptr;
    const double *Dd = nullptr;
    double *alpha = nullptr;
    int sub = 0;   // index into e2_sub / sc2_sub (0 = A, 2 = C)
    int isym = 1;  // symmetry block
};

// Solve queued Gram blocks (same algebra as solve_gram_block), at most 16 per pass so that the
// K and B' matrices of a pass take distinct eigensolver slots.
static void solve_gram_jobs(Context &c, std::vector<GramJob> &all, double e2_sub[8], double sc2_sub[8]) {
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0);
    for (size_t p0 = 0; p0 < all.size(); p0 += 16) {
        const size_t np = std::min<size_t>(16, all.size() - p0);
        auto nm = [](const char *b, size_t j) { return std::string(b) + "#" + std::to_string(j); };
        std::vector<cplx *> K(np), P(np, nullptr), VC0(np, nullptr), Bp(np, nullptr);
        std::vector<double *> wk(np), wb(np, nullptr), red(np);
        std::vector<int> vlo(np, 0), dimm(np, 0);
        std::vector<EigJob> ek;
        std::vector<bool> chol(np, false), band(np, false);
        std::vector<cplx *> Kc(np, nullptr);
        for (size_t j = 0; j < np; j++) {   // metrics, and (AUTO) their definiteness above the cutoff
            GramJob &g = all[p0 + j];
            K[j] = wsget<cplx>(c, nm("gj.K", j), (size_t)g.Mp * g.Mp);
            gram_metric(c, g.Mp, g.dimn, g.G, K[j]);   // K = G G^H (the metric)
            herm_from_upper(c, g.Mp, K[j], g.Mp);
            if (c.metric_solver == DCG_METRIC_AUTO && g.nouter > 0) {   // kept for the Cholesky route
                Kc[j] = wsget<cplx>(c, nm("gj.Kc", j), (size_t)g.Mp * g.Mp);
                DCG_CUDA(cudaMemcpyAsync(Kc[j], K[j], sizeof(cplx) * (size_t)g.Mp * g.Mp, cudaMemcpyDeviceToDevice,
                                         c.stream));
            }
        }
        for (size_t j = 0; j < np; j++) {
            GramJob &g = all[p0 + j];
            red[j] = nullptr;
            wk[j] = wsget<double>(c, nm("gj.wk", j), g.Mp);
            EigJob e;
            e.n = g.Mp;
            e.A = K[j];
            e.lda = g.Mp;
            e.w = wk[j];
            e.slot = (int)j;
            ek.push_back(e);
        }
        heev_values_batched(c, ek);
        std::vector<std::vector<double>> wh(np);
        for (size_t j = 0; j < np; j++) {
            wh[j].resize(all[p0 + j].Mp);
            DCG_CUDA(cudaMemcpyAsync(wh[j].data(), wk[j], sizeof(double) * wh[j].size(), cudaMemcpyDeviceToHost,
                                     c.stream));
        }
        DCG_CUDA(cudaStreamSynchronize(c.stream));
        std::vector<EigJob> eb;
        std::vector<VecJob> pv;
        for (size_t j = 0; j < np; j++) {
            GramJob &g = all[p0 + j];
            vlo[j] = g.Mp;
            for (int q = 0; q < g.Mp; q++)
                if (wh[j][q] >= 1.0e-8) { vlo[j] = q; break; }   // cutoff.F90:37-70
            dimm[j] = g.Mp - vlo[j];
            if (dimm[j] == 0 || g.nouter == 0) continue;
            if (Kc[j] && vlo[j] <= kWoodburyMaxR) {
                chol[j] = true;
                const double *e2o = nullptr, *sco = nullptr;
                if (vlo[j] == 0) {   // nothing under the cutoff: the Cholesky route
                    gram_cholesky_e2(c, g.Mp, g.dimn, g.G, Kc[j], g.Dd, g.Vsel, g.nouter, g.alpha, (int)j, e2o, sco);
                } else {             // a few under it: deflate them, solve on the complement
                    cplx *Ps = wsget<cplx>(c, nm("gj.Ps", j), (size_t)g.Mp * vlo[j]);
                    heev_vectors_slot(c, (int)j, g.Mp, K[j], g.Mp, 0, vlo[j], Ps, g.Mp);
                    gram_woodbury_e2(c, g.Mp, g.dimn, g.G, Kc[j], Ps, vlo[j], wh[j].back(), g.Dd, g.Vsel, g.nouter,
                                     g.alpha, (int)j, e2o, sco);
                }
                red[j] = wsget<double>(c, nm("gj.red", j), 2);
                dsum(c, e2o, g.nouter, red[j]);
                dsum(c, sco, g.nouter, red[j] + 1);
                continue;
            }
            P[j] = wsget<cplx>(c, nm("gj.P", j), (size_t)g.Mp * dimm[j]);
            VecJob v;
            v.slot = (int)j;
            v.n = v.lda = v.ldz = g.Mp;
            v.A = K[j];
            v.vlo = vlo[j];
            v.vhi = g.Mp;
            v.Z = P[j];
            pv.push_back(v);
        }
        eig_slot_jobs(c, pv, {});   // the kept metric eigenvectors of every block, overlapped
        for (size_t j = 0; j < np; j++) {
            if (!P[j]) continue;
            GramJob &g = all[p0 + j];
            const int dm = dimm[j], Mp = g.Mp;
            cplx *GV = wsget<cplx>(c, nm("gj.GV", j), (size_t)Mp * g.nouter);
            gram_gv(c, Mp, g.nouter, g.dimn, g.G, g.Vsel, GV);
            VC0[j] = wsget<cplx>(c, nm("gj.VC0", j), (size_t)dm * g.nouter);
            gram_phgv(c, dm, g.nouter, Mp, P[j], GV, VC0[j]);
            launch_scale_rows(c, dm, g.nouter, VC0[j], dm, wk[j], vlo[j], true);   // Lambda^-1 P^H G v
            cplx *PD = wsget<cplx>(c, nm("gj.PD", j), (size_t)Mp * dm);
            DCG_CUDA(cudaMemcpyAsync(PD, P[j], sizeof(cplx) * (size_t)Mp * dm, cudaMemcpyDeviceToDevice, c.stream));
            launch_scale_rows(c, Mp, dm, PD, Mp, g.Dd, 0, false);
            Bp[j] = wsget<cplx>(c, nm("gj.Bp", j), (size_t)dm * dm);
            bprime_product(c, Mp, dm, P[j], PD, Bp[j]);   // P^H D P
            herm_from_upper(c, dm, Bp[j], dm);
            wb[j] = wsget<double>(c, nm("gj.wb", j), dm);
            if (tridiag_e2_pays(dm, g.nouter) && band_e2_pays(dm, g.nouter)) {
                band[j] = true;   // E2 from its band form below, no tridiagonal reduction
                continue;
            }
            EigJob e;
            e.n = dm;
            e.A = Bp[j];
            e.lda = dm;
            e.w = wb[j];
            e.slot = (int)(16 + j);
            e.tridiag_only = tridiag_e2_pays(dm, g.nouter);   // E2 from the tridiagonal form
            eb.push_back(e);
        }
        heev_values_batched(c, eb);
        // B' of every block: E2 from the tridiagonal form, or its eigenvectors, overlapped
        std::vector<VecJob> wv;
        std::vector<TE2Job> tv;
        std::vector<cplx *> W(np, nullptr);
        std::vector<double *> e2o(np, nullptr), sco(np, nullptr);
        for (size_t j = 0; j < np; j++) {
            GramJob &g = all[p0 + j];
            if (chol[j] || !Bp[j]) continue;
            const int dm = dimm[j];
            e2o[j] = wsget<double>(c, nm("gj.e2o", j), g.nouter);
            sco[j] = wsget<double>(c, nm("gj.sco", j), g.nouter);
            if (band[j]) {
                band_e2(c, (int)(16 + j), dm, Bp[j], dm, VC0[j], dm, g.nouter, g.alpha, e2o[j], sco[j]);
            } else if (tridiag_e2_pays(dm, g.nouter)) {
                TE2Job t;
                t.slot = (int)(16 + j);
                t.n = dm;
                t.A = Bp[j];
                t.lda = t.ldvc = dm;
                t.VC = VC0[j];
                t.nouter = g.nouter;
                t.alpha = g.alpha;
                t.e2o = e2o[j];
                t.sco = sco[j];
                tv.push_back(t);
            } else {
                W[j] = wsget<cplx>(c, nm("gj.W", j), (size_t)dm * dm);
                VecJob v;
                v.slot = (int)(16 + j);
                v.n = v.lda = v.ldz = dm;
                v.A = Bp[j];
                v.vlo = 0;
                v.vhi = dm;
                v.Z = W[j];
                wv.push_back(v);
            }
        }
        eig_slot_jobs(c, wv, tv);
        for (size_t j = 0; j < np; j++) {
            GramJob &g = all[p0 + j];
            if (chol[j] || !Bp[j]) continue;
            const int dm = dimm[j];
            if (W[j]) {
                cplx *VC1 = wsget<cplx>(c, nm("gj.VC1", j), (size_t)dm * g.nouter);
                zgemm(c, OP_C, OP_N, dm, g.nouter, dm, one, W[j], dm, 0, VC0[j], dm, 0, zero, VC1, dm, 0, 1);
                launch_e2(c, VC1, dm, g.nouter, g.alpha, wb[j], e2o[j], sco[j]);
            }
            red[j] = wsget<double>(c, nm("gj.red", j), 2);
            dsum(c, e2o[j], g.nouter, red[j]);
            dsum(c, sco[j], g.nouter, red[j] + 1);
        }
        std::vector<double> hr(2 * np, 0.0);
        for (size_t j = 0; j < np; j++)
            if (red[j]) DCG_CUDA(cudaMemcpyAsync(&hr[2 * j], red[j], 2 * sizeof(double), cudaMemcpyDeviceToHost, c.stream));
        DCG_CUDA(cudaStreamSynchronize(c.stream));
        for (size_t j = 0; j < np; j++) {
            e2_sub[all[p0 + j].sub] += hr[2 * j];
            sc2_sub[all[p0 + j].sub] += hr[2 * j + 1];
            sym_record(c, all[p0 + j].sub, all[p0 + j].isym, hr[2 * j], hr[2 * j + 1], dimm[j]);
        }
    }
}

// run the per-isym blocks of one subspace; V is the full V tensor on the device
static void run_blocks(SubCtx &sc, char sub, const cplx *V, std::vector<BlockSpec> &blocks, double &e2, double &sc2) {
    Context &c = *sc.c;
    e2 = 0.0;
    sc2 = 0.0;
    // Gram route for A (nelec+1 electrons) and C (nelec-1): taken for a block whose dimension
    // exceeds the number of determinants of that space
    const bool gram_kind = (sub == 'A' || sub == 'C') && sc.Y != nullptr;
    const int ne_p = sub == 'A' ? c.ne + 1 : c.ne - 1;
    std::vector<uint64_t> dets_p;
    if (gram_kind) dets_p = gosper_all(c.na, ne_p);
    const int Mp = (int)dets_p.size();
    uint64_t *d_dets_p = nullptr;
    double *d_Dp = nullptr;
    const std::string sfx(1, sub);
    for (size_t bi = 0; bi < blocks.size(); bi++) {
        BlockSpec &b = blocks[bi];
        if (b.dimn == 0) continue;
        const int nouter = (int)b.outer_off.size();
        if (gram_kind && b.dimn > Mp) {
            if (Mp == 0) continue;   // S = 0: no kept vector, nothing printed
            if (!d_dets_p) {
                std::vector<double> Dp(Mp);
                for (int r = 0; r < Mp; r++) {
                    double e = 0.0;
                    for (int w = 0; w < c.na; w++)
                        if ((dets_p[r] >> w) & 1ull) e += sc.eps[c.ni + w];
                    Dp[r] = e;
                }
                d_dets_p = upload(c, "gram.dets" + sfx, dets_p);
                d_Dp = upload(c, "gram.D" + sfx, Dp);
            }
            if (nouter == 0) {   // no contribution; the kept count of K = G G^H decides the print
                int *ind = upload(c, "blk.ind", b.ind);
                cplx *G = wsget<cplx>(c, "gram.G", (size_t)Mp * b.dimn);
                launch_gram(c, c.na, Mp, d_dets_p, sc.M, sc.Y, ind, b.dimn, sub == 'A' ? 1 : 0, G);
                cplx *K = wsget<cplx>(c, "gram.Kcount", (size_t)Mp * Mp);
                gram_metric(c, Mp, b.dimn, G, K);
                sym_record(c, sub - 'A', b.isym, 0.0, 0.0, kept_count(c, Mp, K, Mp));
                continue;
            }
            if (sc.jobs) {   // queue for the joint A/C solve: buffers named per job
                const std::string jn = sfx + std::to_string(bi);
                int *ind = upload(c, "gq.ind" + jn, b.ind);
                GramJob g;
                g.Mp = Mp;
                g.dimn = b.dimn;
                g.nouter = nouter;
                g.G = wsget<cplx>(c, "gq.G" + jn, (size_t)Mp * b.dimn);
                launch_gram(c, c.na, Mp, d_dets_p, sc.M, sc.Y, ind, b.dimn, sub == 'A' ? 1 : 0, g.G);
                int64_t *oo = upload(c, "gq.oo" + jn, b.outer_off);
                int64_t *io = upload(c, "gq.io" + jn, b.inner_off);
                g.alpha = upload(c, "gq.alpha" + jn, b.alpha);
                g.Vsel = wsget<cplx>(c, "gq.Vsel" + jn, (size_t)b.dimn * nouter);
                launch_gather_v(c, V, oo, nouter, io, b.dimn, g.Vsel);
                g.Dd = d_Dp;
                g.sub = sub == 'A' ? 0 : 2;
                g.isym = b.isym;
                sc.jobs->push_back(g);
                continue;
            }
            int *ind = upload(c, "blk.ind", b.ind);
            cplx *G = wsget<cplx>(c, "gram.G", (size_t)Mp * b.dimn);
            launch_gram(c, c.na, Mp, d_dets_p, sc.M, sc.Y, ind, b.dimn, sub == 'A' ? 1 : 0, G);
            int64_t *oo = upload(c, "blk.oo", b.outer_off);
            int64_t *io = upload(c, "blk.io", b.inner_off);
            double *al = upload(c, "blk.alpha", b.alpha);
            cplx *Vsel = wsget<cplx>(c, "blk.Vsel", (size_t)b.dimn * nouter);
            launch_gather_v(c, V, oo, nouter, io, b.dimn, Vsel);
            BlockOut o = solve_gram_block(c, Mp, b.dimn, G, d_Dp, Vsel, nouter, al);
            e2 += o.e2;
            sc2 += o.sc2;
            sym_record(c, sub - 'A', b.isym, o.e2, o.sc2, o.dimm);
            continue;
        }
        if (nouter == 0) {   // no contribution; the kept count of S decides the print
            int *ind = upload(c, "blk.ind", b.ind);
            cplx *S = wsget<cplx>(c, "blk.S", (size_t)b.dimn * b.dimn);
            cplx *B = wsget<cplx>(c, "blk.B", (size_t)b.dimn * b.dimn);
            launch_SB(c, sub, sc.rv, ind, b.dimn, sc.eps_act_d, sc.e0, S, B);
            sym_record(c, sub - 'A', b.isym, 0.0, 0.0, kept_count(c, b.dimn, S, b.dimn));
            continue;
        }
        if (sc.bjobs) {   // queue for the joint solve of the S/B-route blocks
            const std::string jn = std::string(1, sub) + std::to_string(bi);
            int *ind = upload(c, "bq.ind" + jn, b.ind);
            BlockJob j;
            j.sub = sub - 'A';
            j.isym = b.isym;
            j.dimn = b.dimn;
            j.nouter = nouter;
            j.S = wsget<cplx>(c, "bq.S" + jn, (size_t)b.dimn * b.dimn);
            j.B = wsget<cplx>(c, "bq.B" + jn, (size_t)b.dimn * b.dimn);
            launch_SB(c, sub, sc.rv, ind, b.dimn, sc.eps_act_d, sc.e0, j.S, j.B);
            int64_t *oo = upload(c, "bq.oo" + jn, b.outer_off);
            int64_t *io = upload(c, "bq.io" + jn, b.inner_off);
            j.alpha = upload(c, "bq.alpha" + jn, b.alpha);
            j.Vsel = wsget<cplx>(c, "bq.Vsel" + jn, (size_t)b.dimn * nouter);
            launch_gather_v(c, V, oo, nouter, io, b.dimn, j.Vsel);
            sc.bjobs->push_back(j);
            continue;
        }
        int *ind = upload(c, "blk.ind", b.ind);
        cplx *S = wsget<cplx>(c, "blk.S", (size_t)b.dimn * b.dimn);
        cplx *B = wsget<cplx>(c, "blk.B", (size_t)b.dimn * b.dimn);
        launch_SB(c, sub, sc.rv, ind, b.dimn, sc.eps_act_d, sc.e0, S, B);
        int64_t *oo = upload(c, "blk.oo", b.outer_off);
        int64_t *io = upload(c, "blk.io", b.inner_off);
        double *al = upload(c, "blk.alpha", b.alpha);
        cplx *Vsel = wsget<cplx>(c, "blk.Vsel", (size_t)b.dimn * nouter);
        launch_gather_v(c, V, oo, nouter, io, b.dimn, Vsel);
        BlockOut o = solve_block(c, b.dimn, S, B, Vsel, nouter, al);
        e2 += o.e2;
        sc2 += o.sc2;
        sym_record(c, sub - 'A', b.isym, o.e2, o.sc2, o.dimm);
    }
}

static inline int kp(int x) { return (x % 2 == 1) ? x + 1 : x - 1; }

// First index whose value is within a relative 1e-8 of the maximum.
static int first_near_max(const std::vector<double> &x) {
    double m = x[0];
    for (double v : x) m = std::max(m, v);
    for (size_t i = 0; i < x.size(); i++)
        if (x[i] >= m - 1e-8 * std::fabs(m)) return (int)i;
    return 0;
}

// Canonical vectors inside exactly degenerate eigenvalue pairs of the active Fock block.
// ZHEEV's choice inside a degenerate pair is decided by rounding and the reference's
// complex E-space V build (solve_E_subspace.F90 vEmat_complex, dim1_density(it,k)) is not
// invariant under it; this picks one of those equally valid choices deterministically:
// v1 = P e_k/|P e_k| with k the first index of near-maximal P_kk (P the pair projector),
// v2 the orthogonal unit vector of the pair with its first near-largest component real
// positive.  V is n x n column-major.
static void canonical_pairs(int n, const std::vector<double> &w, std::vector<cplx> &V) {
    int q = 0;
    while (q < n - 1) {
        if (std::fabs(w[q + 1] - w[q]) > 1e-10 * std::max(1.0, std::fabs(w[q]))) {
            q++;
            continue;
        }
        cplx *c0 = V.data() + (size_t)n * q, *c1 = V.data() + (size_t)n * (q + 1);
        std::vector<double> pk(n);
        for (int r = 0; r < n; r++) pk[r] = cabs2(c0[r]) + cabs2(c1[r]);
        const int k = first_near_max(pk);
        cplx a0 = cconj(c0[k]), a1 = cconj(c1[k]);
        const double na = std::sqrt(cabs2(a0) + cabs2(a1));
        a0 = cscale(a0, 1.0 / na);
        a1 = cscale(a1, 1.0 / na);
        const cplx b0 = mk(-a1.x, a1.y), b1 = cconj(a0);   // (-conj(a1), conj(a0))
        std::vector<cplx> v1(n), v2(n);
        std::vector<double> m2(n);
        for (int r = 0; r < n; r++) {
            v1[r] = cadd(cmul(c0[r], a0), cmul(c1[r], a1));
            v2[r] = cadd(cmul(c0[r], b0), cmul(c1[r], b1));
            m2[r] = std::sqrt(cabs2(v2[r]));
        }
        const int l = first_near_max(m2);
        const cplx ph = cscale(cconj(v2[l]), 1.0 / m2[l]);
        for (int r = 0; r < n; r++) {
            c0[r] = v1[r];
            c1[r] = cmul(v2[r], ph);
        }
        q += 2;
    }
}

}  // namespace dcg

namespace dcg {

static int caspt2(Context &c, uint32_t skip, double e2_sub[8], double sc2_sub[8], double *e0_out, double *et_out) {
    if (!c.have_casci) throw Error{DCG_E_STATE, "dcg_caspt2 before dcg_casci"};
    c.gram_cholesky_blocks = 0;
    c.gram_woodbury_blocks = 0;
    DevSystem &d = dev(c);
    const int ni = c.ni, na = c.na, ns = c.ns, nmoc = ni + na;
    const cplx one = mk(1.0, 0.0), zero = mk(0.0, 0.0), mone = mk(-1.0, 0.0);
    for (int k = 0; k < 8; k++) { e2_sub[k] = 0.0; sc2_sub[k] = 0.0; }
    c.sym_e2.assign((size_t)8 * c.nsym, 0.0);
    c.sym_sc2.assign((size_t)8 * c.nsym, 0.0);
    c.sym_printed.assign((size_t)8 * c.nsym, 0);
    if (ni == 0 && ns == 0) throw Error{DCG_E_ARG, "CASPT2 energy undefined for ninact = 0 and nsec = 0"};
    if (c.precision == DCG_PREC_SPLIT) split_reset(c);

    // full N-electron space and the CI-space positions inside it
    std::vector<uint64_t> full = gosper_all(na, c.ne);
    const int64_t M = (int64_t)full.size();
    std::vector<int64_t> pos(d.ndet);
    for (int i = 0; i < d.ndet; i++)
        pos[i] = std::lower_bound(full.begin(), full.end(), c.dets[i]) - full.begin();
    uint64_t *d_full = upload(c, "pt.full", full);
    int64_t *d_pos = upload(c, "pt.pos", pos);
    cplx *psi = wsget<cplx>(c, "pt.psi", M);

    // ---- Fock matrix of the CASCI state (fockcasci.F90:4-90) and its diagonalisation
    stage_begin(c, ST_FOCK);
    launch_embed(c, d.ndet, d_pos, d.c0, psi, M);
    RdmBufs r0 = rdm_build(c, d_full, M, psi, nullptr, false);
    cplx *f = wsget<cplx>(c, "pt.f", (size_t)c.nmo * c.nmo);
    launch_fock(c, d.h, d.inttw, d.cls, r0.g1, f);
    // fockdiag.F90:4-78 / cdiag0 (diag.F90:230-375): per space and irrep
    cplx *U = wsget<cplx>(c, "pt.U", (size_t)c.nmo * c.nmo);
    DCG_CUDA(cudaMemsetAsync(U, 0, sizeof(cplx) * (size_t)c.nmo * c.nmo, c.stream));
    c.eps.assign(c.nmo, 0.0);
    const int rng[3][2] = {{0, ni}, {ni, nmoc}, {nmoc, nmoc + ns}};
    // the per-space, per-irrep blocks are independent: their reductions run in batched
    // launches (at most kEigSlots at a time), then each block's vectors are formed
    struct FockBlk {
        int sp;
        std::vector<int> ind;
        int *dind;
        cplx *blk, *vec;
        double *w;
    };
    std::vector<FockBlk> fb;
    for (int sp = 0; sp < 3; sp++)
        for (int sym = 1; sym <= c.nsym; sym++) {
            FockBlk b;
            b.sp = sp;
            for (int i = rng[sp][0]; i < rng[sp][1]; i++)
                if (c.irpamo[i] == sym) b.ind.push_back(i);
            if (!b.ind.empty()) fb.push_back(b);
        }
    for (size_t b0 = 0; b0 < fb.size(); b0 += kEigSlots) {
        const size_t nbat = std::min<size_t>(kEigSlots, fb.size() - b0);
        std::vector<EigJob> jobs;
        for (size_t q = 0; q < nbat; q++) {
            FockBlk &b = fb[b0 + q];
            const int nb = (int)b.ind.size();
            const std::string t = "#" + std::to_string(q);
            b.dind = upload(c, "fd.ind" + t, b.ind);
            b.blk = wsget<cplx>(c, "fd.blk" + t, (size_t)nb * nb);
            b.vec = wsget<cplx>(c, "fd.vec" + t, (size_t)nb * nb);
            b.w = wsget<double>(c, "fd.w" + t, nb);
            launch_gather2(c, f, c.nmo, b.dind, nb, b.blk);
            EigJob e;
            e.n = nb;
            e.A = b.blk;
            e.lda = nb;
            e.w = b.w;
            e.slot = (int)q;
            jobs.push_back(e);
        }
        heev_values_batched(c, jobs);
        std::vector<VecJob> vj;
        for (size_t q = 0; q < nbat; q++) {
            FockBlk &b = fb[b0 + q];
            VecJob v;
            v.slot = (int)q;
            v.n = v.lda = v.ldz = v.vhi = (int)b.ind.size();
            v.A = b.blk;
            v.Z = b.vec;
            vj.push_back(v);
        }
        eig_slot_jobs(c, vj, {});
        for (size_t q = 0; q < nbat; q++) {
            FockBlk &b = fb[b0 + q];
            const int nb = (int)b.ind.size();
            std::vector<double> wh = download(c, b.w, nb);
            if (b.sp == 1) {   // active space: canonical vectors inside degenerate pairs
                std::vector<cplx> vh = download(c, b.vec, (size_t)nb * nb);
                canonical_pairs(nb, wh, vh);
                DCG_CUDA(cudaMemcpyAsync(b.vec, vh.data(), sizeof(cplx) * vh.size(), cudaMemcpyHostToDevice,
                                         c.stream));
                DCG_CUDA(cudaStreamSynchronize(c.stream));
            }
            launch_scatter2(c, b.vec, nb, b.dind, U, c.nmo);
            for (int k = 0; k < nb; k++) c.eps[b.ind[k]] = wh[k];
        }
    }
    d.eps = upload(c, "pt.eps", c.eps);
    stage_end(c, ST_FOCK);

    // ---- CI rotation into the new active spinors (trac.F90:76-156)
    stage_begin(c, ST_CIROT);
    cplx *Uact = wsget<cplx>(c, "pt.Uact", (size_t)na * na + 1);
    if (na > 0)
        DCG_CUDA(cudaMemcpy2DAsync(Uact, na * sizeof(cplx), U + ni + (size_t)c.nmo * ni, c.nmo * sizeof(cplx),
                                   na * sizeof(cplx), na, cudaMemcpyDeviceToDevice, c.stream));
    cplx *ds = wsget<cplx>(c, "pt.ds", (size_t)d.ndet * d.ndet);
    cplx *c1 = wsget<cplx>(c, "pt.c1", d.ndet);
    if ((int64_t)d.ndet == M && na > 0) {
        // Full determinant space: ds(U)(k, l) = det U[occ_k, occ_l] is the ne-th exterior power
        // of the unitary U, and exterior powers multiply (Cauchy-Binet), so ds(U)^-1 = ds(U^H):
        // c1 = ds(U^H) c0 solves the reference's ZGESV system without a factorisation.
        std::vector<cplx> uh = download(c, Uact, (size_t)na * na), uht((size_t)na * na);
        for (int i = 0; i < na; i++)
            for (int j = 0; j < na; j++) uht[j + (size_t)na * i] = cconj(uh[i + (size_t)na * j]);
        cplx *UactH = upload(c, "pt.UactH", uht);
        launch_detsc(c, d.dets, d.ndet, UactH, ds);
        zgemm(c, OP_N, OP_N, d.ndet, 1, d.ndet, one, ds, d.ndet, 0, d.c0, d.ndet, 0, zero, c1, d.ndet, 0, 1);
    } else {
        // restricted (RAS or symmetry) determinant list: the reference's linear solve
        launch_detsc(c, d.dets, d.ndet, Uact, ds);
        DCG_CUDA(cudaMemcpyAsync(c1, d.c0, sizeof(cplx) * d.ndet, cudaMemcpyDeviceToDevice, c.stream));
        const int info = zgesv(c, d.ndet, ds, d.ndet, c1);
        if (info != 0)
            throw Error{info, "CI rotation: singular determinant-overlap matrix (ZGESV info " + std::to_string(info) + ")"};
    }
    stage_end(c, ST_CIROT);

    // ---- densities of the rotated state and e0 (calce0.F90:4-50)
    stage_begin(c, ST_RDM);
    launch_embed(c, d.ndet, d_pos, c1, psi, M);
    const double *eps_act_d = d.eps + ni;
    const bool need3 = (ni > 0) || (ns > 0);
    RdmBufs rd = rdm_build(c, d_full, M, psi, eps_act_d, need3);
    std::vector<cplx> d1h = download(c, rd.g1, (size_t)na * na);
    double e0 = 0.0;
    for (int w = 0; w < na; w++) e0 += d1h[w + (size_t)na * w].x * c.eps[ni + w];
    stage_end(c, ST_RDM);

    // ---- effective one-electron terms and transformed integral classes
    stage_begin(c, ST_TRANS);
    cplx *Ui = wsget<cplx>(c, "pt.Ui", (size_t)ni * ni + 1);
    cplx *Ua = wsget<cplx>(c, "pt.Ua", (size_t)na * na + 1);
    cplx *Us = wsget<cplx>(c, "pt.Us", (size_t)ns * ns + 1);
    if (ni) DCG_CUDA(cudaMemcpy2DAsync(Ui, ni * sizeof(cplx), U, c.nmo * sizeof(cplx), ni * sizeof(cplx), ni, cudaMemcpyDeviceToDevice, c.stream));
    if (na) DCG_CUDA(cudaMemcpyAsync(Ua, Uact, sizeof(cplx) * na * na, cudaMemcpyDeviceToDevice, c.stream));
    if (ns) DCG_CUDA(cudaMemcpy2DAsync(Us, ns * sizeof(cplx), U + nmoc + (size_t)c.nmo * nmoc, c.nmo * sizeof(cplx), ns * sizeof(cplx), ns, cudaMemcpyDeviceToDevice, c.stream));
    const cplx *Usp[4] = {nullptr, Ui, Ua, Us};
    // core Fock pieces -> effh blocks: effh = U_p^H F U_q
    cplx *Fai = wsget<cplx>(c, "pt.Fai", (size_t)na * ni + 1);
    cplx *Fsi = wsget<cplx>(c, "pt.Fsi", (size_t)ns * ni + 1);
    cplx *Fsa = wsget<cplx>(c, "pt.Fsa", (size_t)ns * na + 1);
    launch_core_fock(c, d.h, d.inttw, d.cls, Fai, Fsi, Fsa);
    cplx *tmp2 = wsget<cplx>(c, "pt.tmp2", (size_t)std::max({na * ni, ns * ni, ns * na, 1}));
    cplx *effA = wsget<cplx>(c, "pt.effA", (size_t)na * ni + 1);
    cplx *effD = wsget<cplx>(c, "pt.effD", (size_t)ns * ni + 1);
    cplx *effC = wsget<cplx>(c, "pt.effC", (size_t)ns * na + 1);
    auto sandwich = [&](const cplx *Up, int np, const cplx *Fm, const cplx *Uq, int nq, cplx *out) {
        if (np == 0 || nq == 0) return;
        zgemm(c, OP_N, OP_N, np, nq, nq, one, Fm, np, 0, Uq, nq, 0, zero, tmp2, np, 0, 1);
        zgemm(c, OP_C, OP_N, np, nq, np, one, Up, np, 0, tmp2, np, 0, zero, out, np, 0, 1);
    };
    sandwich(Ua, na, Fai, Ui, ni, effA);
    sandwich(Us, ns, Fsi, Ui, ni, effD);
    sandwich(Us, ns, Fsa, Ua, na, effC);
    launch_zero_small(c, effC, (int64_t)ns * na, 1.0e-10);   // vCmat: |effh| < 1e-10 skipped
    // transformed classes
    size_t maxsz = 1;
    for (int id = 0; id < CL_COUNT; id++) maxsz = std::max(maxsz, (size_t)d.cls[id].size);
    const size_t szA1 = (size_t)na * ni * na * na, szB = (size_t)na * ni * na * ni;
    maxsz = std::max({maxsz, szA1, szB});
    cplx *ttmp = wsget<cplx>(c, "pt.ttmp", maxsz);
    cplx *orig = wsget<cplx>(c, "pt.orig", std::max(szA1, szB) + 1);
    auto tr_class = [&](const char *name, const cplx *src, const int sp[4], const int dm[4]) -> cplx * {
        const size_t sz = (size_t)dm[0] * dm[1] * dm[2] * dm[3];
        cplx *out = wsget<cplx>(c, std::string("tr.") + name, sz + 1);
        const cplx *Ux[4] = {Usp[sp[0]], Usp[sp[1]], Usp[sp[2]], Usp[sp[3]]};
        FamScope fs(c, DCG_FAM_TRANSFORM, 8.0 * (double)sz * (dm[0] + dm[1] + dm[2] + dm[3]));
        nvtxRangePushA((std::string("tr_") + name).c_str());
        transform4(c, src, out, ttmp, dm, Ux);
        nvtxRangePop();
        return out;
    };
    auto tr_id = [&](const char *name, int id) -> cplx * { return tr_class(name, d.cls[id].p, d.cls[id].sp, d.cls[id].dim); };
    stage_end(c, ST_TRANS);

    SubCtx sc;
    sc.c = &c;
    sc.rv = rd.view;
    sc.eps_act_d = eps_act_d;
    sc.eps = c.eps;
    sc.e0 = e0;
    sc.Y = rd.Y;
    sc.M = rd.M;
    const double es = c.eshift;
    auto irp = [&](int g) { return c.irpamo[g]; };
    const bool c1sym = (c.nsym == 1);
    auto timed = [&](int st, auto fn) { stage_begin(c, st); fn(); stage_end(c, st); };

    std::vector<GramJob> gjobs;   // A and C Gram blocks, solved together after C's build
    sc.jobs = &gjobs;

    // ================= A: E_ti E_uv|0>  (solve_A_subspace.F90:26-678)
    if (ni > 0 && !(skip & 1u)) timed(ST_A, [&] {
        stage_begin(c, ST_TRANS);
        const int off[4] = {ni, 0, ni, ni}, dm[4] = {na, ni, na, na}, sp[4] = {2, 1, 2, 2};
        launch_subblock(c, d.inttw, nmoc, off, dm, orig);
        cplx *A1 = tr_class("A1", orig, sp, dm);
        stage_end(c, ST_TRANS);
        const int64_t n3 = (int64_t)na * na * na;
        cplx *V = wsget<cplx>(c, "v.A", (size_t)ni * n3 + 1);
        cplx *A1p = wsget<cplx>(c, "v.A1p", (size_t)ni * n3 + 1);
        cplx *P3 = wsget<cplx>(c, "v.P3", (size_t)n3 * n3 + 1);
        launch_permute_A1(c, A1, na, ni, A1p);
        launch_perm_A(c, sc.rv, P3, nullptr);
        zgemm(c, OP_N, OP_N, ni, (int)n3, (int)n3, mone, A1p, ni, 0, P3, n3, 0, zero, V, ni, 0, 1);
        launch_v_A_rest(c, sc.rv, A1, effA, ni, V);
        std::vector<BlockSpec> blocks;
        for (int isym = 1; isym <= c.nsym; isym++) {
            BlockSpec b;
            b.isym = isym;
            for (int x = 0; x < na; x++)
                for (int y = 0; y < na; y++)
                    for (int z = 0; z < na; z++)
                        if (c1sym || c.ms(c.md(irp(ni + x), isym), c.md(irp(ni + y), irp(ni + z))) == 1) {
                            b.ind.push_back(x); b.ind.push_back(y); b.ind.push_back(z);
                            b.inner_off.push_back((int64_t)ni * (x + (int64_t)na * (y + (int64_t)na * z)));
                        }
            b.dimn = (int)b.inner_off.size();
            for (int i = 0; i < ni; i++)
                if (c1sym || irp(i) == isym) {
                    b.outer_off.push_back(i);
                    b.alpha.push_back(-c.eps[i] - e0 + es);
                }
            blocks.push_back(b);
        }
        run_blocks(sc, 'A', V, blocks, e2_sub[0], sc2_sub[0]);
    });

    // the S/B-route blocks of B .. G are queued and solved together after G
    std::vector<BlockJob> bjobs;
    sc.bjobs = &bjobs;

    // ================= B: E_ti E_uj|0>, t>u, i>j  (solve_B_subspace.F90:27-591)
    if (ni > 0 && !(skip & 2u)) timed(ST_B, [&] {
        stage_begin(c, ST_TRANS);
        const int off[4] = {ni, 0, ni, 0}, dm[4] = {na, ni, na, ni}, sp[4] = {2, 1, 2, 1};
        launch_subblock(c, d.inttw, nmoc, off, dm, orig);
        cplx *Bc = tr_class("B", orig, sp, dm);
        stage_end(c, ST_TRANS);
        const int np = ni * (ni - 1) / 2;
        cplx *V = wsget<cplx>(c, "v.B", (size_t)np * na * na + 1);
        launch_v_B(c, sc.rv, Bc, ni, V);
        std::vector<BlockSpec> blocks;
        for (int isym = 1; isym <= c.nsym; isym++) {
            BlockSpec b;
            b.isym = isym;
            for (int t = 0; t < na; t++)
                for (int u = 0; u < t; u++)
                    if (c1sym || c.md(irp(ni + t), kp(irp(ni + u))) == isym) {
                        b.ind.push_back(t); b.ind.push_back(u);
                        b.inner_off.push_back((int64_t)np * (t + (int64_t)na * u));
                    }
            b.dimn = (int)b.inner_off.size();
            for (int i = 0; i < ni; i++)
                for (int j = 0; j < i; j++)
                    if (c1sym || c.ms(c.md(kp(irp(i)), irp(j)), isym) == 1) {
                        b.outer_off.push_back((int64_t)i * (i - 1) / 2 + j);
                        b.alpha.push_back(-c.eps[i] - c.eps[j] - e0 + es);
                    }
            blocks.push_back(b);
        }
        run_blocks(sc, 'B', V, blocks, e2_sub[1], sc2_sub[1]);
    });

    // ================= C: E_at E_uv|0>  (solve_C_subspace.F90:26-658)
    if (ns > 0 && !(skip & 4u)) timed(ST_C, [&] {
        stage_begin(c, ST_TRANS);
        cplx *C1 = tr_id("C1", CL_C1);
        stage_end(c, ST_TRANS);
        const int64_t n3 = (int64_t)na * na * na;
        cplx *V = wsget<cplx>(c, "v.C", (size_t)ns * n3 + 1);
        cplx *P3 = wsget<cplx>(c, "v.P3", (size_t)n3 * n3 + 1);
        cplx *P2 = wsget<cplx>(c, "v.P2", (size_t)na * n3 + 1);
        launch_perm_C2(c, sc.rv, P3, P2);
        // V = C1 P3 + effh P2: its errors stay relative through X^H V, so the large product may
        // run on the split-precision tensor cores
        if (c.precision == DCG_PREC_SPLIT)
            zgemm_split(c, ns, (int)n3, (int)n3, 1, C1, 1, ns, 0, P3, n3, 0, V, 1, ns, 0, false, c.split_lbo,
                        c.split_sbo);
        else
            zgemm(c, OP_N, OP_N, ns, (int)n3, (int)n3, one, C1, ns, 0, P3, n3, 0, zero, V, ns, 0, 1);
        zgemm(c, OP_N, OP_N, ns, (int)n3, na, one, effC, ns, 0, P2, na, 0, one, V, ns, 0, 1);
        std::vector<BlockSpec> blocks;
        for (int isym = 1; isym <= c.nsym; isym++) {
            BlockSpec b;
            b.isym = isym;
            for (int x = 0; x < na; x++)
                for (int y = 0; y < na; y++)
                    for (int z = 0; z < na; z++)
                        if (c1sym || c.ms(c.md(isym, irp(ni + x)), c.md(irp(ni + y), irp(ni + z))) == 1) {
                            b.ind.push_back(x); b.ind.push_back(y); b.ind.push_back(z);
                            b.inner_off.push_back((int64_t)ns * (x + (int64_t)na * (y + (int64_t)na * z)));
                        }
            b.dimn = (int)b.inner_off.size();
            for (int a = 0; a < ns; a++)
                if (c1sym || irp(nmoc + a) == isym) {
                    b.outer_off.push_back(a);
                    b.alpha.push_back(c.eps[nmoc + a] - e0 + es);
                }
            blocks.push_back(b);
        }
        run_blocks(sc, 'C', V, blocks, e2_sub[2], sc2_sub[2]);
    });
    // joint solve of the queued A and C Gram blocks (their eigenproblems batched)
    if (!gjobs.empty()) timed(ST_AC, [&] { solve_gram_jobs(c, gjobs, e2_sub, sc2_sub); });
    sc.jobs = nullptr;

    // ================= D: E_ai E_tu|0>  (solve_D_subspace.F90:25-609)
    if (ni > 0 && ns > 0 && !(skip & 8u)) timed(ST_D, [&] {
        stage_begin(c, ST_TRANS);
        cplx *D1c = tr_id("D1", CL_D1);
        cplx *D2c = tr_id("D2", CL_D2);
        stage_end(c, ST_TRANS);
        const int64_t nsi = (int64_t)ns * ni;
        cplx *V = wsget<cplx>(c, "v.D", (size_t)nsi * na * na + 1);
        launch_v_D(c, sc.rv, D1c, D2c, effD, ni, ns, V);
        std::vector<BlockSpec> blocks;
        for (int isym = 1; isym <= c.nsym; isym++) {
            BlockSpec b;
            b.isym = isym;
            for (int t = 0; t < na; t++)
                for (int u = 0; u < na; u++)
                    if (c1sym || c.md(irp(ni + t), irp(ni + u)) == isym) {
                        b.ind.push_back(t); b.ind.push_back(u);
                        b.inner_off.push_back(nsi * (t + (int64_t)na * u));
                    }
            b.dimn = (int)b.inner_off.size();
            for (int a = 0; a < ns; a++)
                for (int i = 0; i < ni; i++)
                    if (c1sym || c.ms(c.md(irp(nmoc + a), irp(i)), isym) == 1) {
                        b.outer_off.push_back(a + (int64_t)ns * i);
                        b.alpha.push_back(c.eps[nmoc + a] - c.eps[i] - e0 + es);
                    }
            blocks.push_back(b);
        }
        run_blocks(sc, 'D', V, blocks, e2_sub[3], sc2_sub[3]);
    });

    // ================= E: E_ti E_aj|0>, i>j  (solve_E_subspace.F90:26-476)
    if (ni > 0 && ns > 0 && !(skip & 16u)) timed(ST_E, [&] {
        stage_begin(c, ST_TRANS);
        cplx *Ec = tr_id("E", CL_E);
        stage_end(c, ST_TRANS);
        const int np = ni * (ni - 1) / 2;
        const int64_t nq = (int64_t)ns * np;
        cplx *V = wsget<cplx>(c, "v.E", (size_t)nq * na + 1);
        launch_v_E(c, sc.rv, Ec, ni, ns, V);
        std::vector<BlockSpec> blocks;
        for (int isym = 1; isym <= c.nsym; isym++) {
            BlockSpec b;
            b.isym = isym;
            for (int t = 0; t < na; t++)
                if (irp(ni + t) == isym) {
                    b.ind.push_back(t);
                    b.inner_off.push_back(nq * t);
                }
            b.dimn = (int)b.inner_off.size();
            for (int i = 0; i < ni; i++)
                for (int j = 0; j < i; j++)
                    for (int a = 0; a < ns; a++)
                        if (c1sym || c.ms(c.md(isym, irp(i)), c.md(irp(nmoc + a), irp(j))) == 1) {
                            b.outer_off.push_back(a + (int64_t)ns * ((int64_t)i * (i - 1) / 2 + j));
                            b.alpha.push_back(c.eps[nmoc + a] - c.eps[i] - c.eps[j] - e0 + es);
                        }
            blocks.push_back(b);
        }
        run_blocks(sc, 'E', V, blocks, e2_sub[4], sc2_sub[4]);
    });

    // ================= F: E_at E_bu|0>, a>b, t>u  (solve_F_subspace.F90:26-544)
    if (ns > 0 && !(skip & 32u)) timed(ST_F, [&] {
        stage_begin(c, ST_TRANS);
        cplx *Fc = tr_id("F", CL_F);
        stage_end(c, ST_TRANS);
        const int64_t ns2 = (int64_t)ns * ns, na2 = (int64_t)na * na;
        cplx *Fp = wsget<cplx>(c, "v.Fp", (size_t)ns2 * na2 + 1);
        cplx *P2 = wsget<cplx>(c, "v.P2F", (size_t)na2 * na2 + 1);
        cplx *V = wsget<cplx>(c, "v.F", (size_t)ns2 * na2 + 1);
        launch_F_pack(c, Fc, ns, na, Fp);
        launch_perm_F(c, sc.rv, P2, nullptr);
        if (c.precision == DCG_PREC_SPLIT)
            zgemm_split(c, (int)ns2, (int)na2, (int)na2, 1, Fp, 1, ns2, 0, P2, na2, 0, V, 1, ns2, 0, false,
                        c.split_lbo, c.split_sbo);
        else
            zgemm(c, OP_N, OP_N, (int)ns2, (int)na2, (int)na2, one, Fp, ns2, 0, P2, na2, 0, zero, V, ns2, 0, 1);
        std::vector<BlockSpec> blocks;
        for (int isym = 1; isym <= c.nsym; isym++) {
            BlockSpec b;
            b.isym = isym;
            for (int t = 0; t < na; t++)
                for (int u = 0; u < t; u++)
                    if (c1sym || c.md(kp(irp(ni + u)), irp(ni + t)) == isym) {
                        b.ind.push_back(t); b.ind.push_back(u);
                        b.inner_off.push_back(ns2 * (t + (int64_t)na * u));
                    }
            b.dimn = (int)b.inner_off.size();
            for (int a = 0; a < ns; a++)
                for (int bb = 0; bb < a; bb++)
                    if (c1sym || c.ms(c.md(irp(nmoc + a), kp(irp(nmoc + bb))), isym) == 1) {
                        b.outer_off.push_back(a + (int64_t)ns * bb);
                        b.alpha.push_back(c.eps[nmoc + a] + c.eps[nmoc + bb] - e0 + es);
                    }
            blocks.push_back(b);
        }
        run_blocks(sc, 'F', V, blocks, e2_sub[5], sc2_sub[5]);
    });

    // ================= G: E_ai E_bt|0>, a>b  (solve_G_subspace.F90:26-469)
    if (ni > 0 && ns > 0 && !(skip & 64u)) timed(ST_G, [&] {
        stage_begin(c, ST_TRANS);
        cplx *Gc = tr_id("G", CL_G);
        stage_end(c, ST_TRANS);
        const int64_t nab = (int64_t)ns * (ns - 1) / 2;
        const int64_t nq = nab * ni;
        cplx *V = wsget<cplx>(c, "v.G", (size_t)nq * na + 1);
        launch_v_G(c, sc.rv, Gc, ni, ns, V);
        std::vector<BlockSpec> blocks;
        for (int isym = 1; isym <= c.nsym; isym++) {
            BlockSpec b;
            b.isym = isym;
            for (int t = 0; t < na; t++)
                if (irp(ni + t) == isym) {
                    b.ind.push_back(t);
                    b.inner_off.push_back(nq * t);
                }
            b.dimn = (int)b.inner_off.size();
            for (int a = 0; a < ns; a++)
                for (int bb = 0; bb < a; bb++)
                    for (int i = 0; i < ni; i++)
                        if (c1sym || c.ms(c.md(irp(nmoc + bb), isym), c.md(irp(nmoc + a), irp(i))) == 1) {
                            b.outer_off.push_back(((int64_t)a * (a - 1) / 2 + bb) + nab * i);
                            b.alpha.push_back(-c.eps[i] + c.eps[nmoc + a] + c.eps[nmoc + bb] - e0 + es);
                        }
            blocks.push_back(b);
        }
        run_blocks(sc, 'G', V, blocks, e2_sub[6], sc2_sub[6]);
    });

    if (!bjobs.empty()) timed(ST_BDEFG, [&] { solve_block_jobs(c, bjobs, e2_sub, sc2_sub); });
    sc.bjobs = nullptr;

    // ================= H: streaming (solve_H_subspace.F90:23-191)
    if (ni > 0 && ns > 0 && !(skip & 128u)) timed(ST_H, [&] {
        stage_begin(c, ST_TRANS);
        cplx *Hc = tr_id("H", CL_H);
        stage_end(c, ST_TRANS);
        const int nblk = h_stream_blocks(ni, ns);
        double *part = wsget<double>(c, "h.part", 2 * (size_t)nblk);
        double *red = wsget<double>(c, "h.red", 2);
        {
            // bytes the kernel must read: both operands of every a > b, i > j pair, the a > b
            // half of the class
            FamScope fs(c, DCG_FAM_HSTREAM, 0.5 * ns * (ns - 1.0) * ni * (ni - 1.0) * sizeof(cplx));
            launch_h_stream2(c, Hc, ni, ns, d.eps, d.eps + nmoc, d.irp, d.irp + nmoc, d.md, d.msy, c.nsym, es, part,
                             part + nblk);
        }
        dsum(c, part, nblk, red);
        dsum(c, part + nblk, nblk, red + 1);
        std::vector<double> hr = download(c, red, 2);
        e2_sub[7] = hr[0];
        sc2_sub[7] = hr[1];
    });

    if (c.precision == DCG_PREC_SPLIT && split_error(c))
        throw Error{DCG_E_NUMERIC, "split-precision GEMM: a pipeline wait timed out"};
    double e2all = 0.0, sumc2 = 0.0;
    for (int k = 0; k < 8; k++) { e2all += e2_sub[k]; sumc2 += sc2_sub[k]; }
    fam_collect(c);
    if (e0_out) *e0_out = e0;
    if (et_out) *et_out = e2all + c.ecas[c.selectroot - 1] - c.eshift * sumc2;   // r4dcaspt2_tra.F90:441
    DCG_CUDA(cudaStreamSynchronize(c.stream));
    return 0;
}

}  // namespace dcg

// ============================================================================ C ABI
using dcg::Context;
using dcg::Error;

#define DCG_API_BODY(ctxp, body)                                                    \
    do {                                                                            \
        if (!(ctxp)) return DCG_E_ARG;                                              \
        Context &c_ = (ctxp)->c;                                                    \
        try {                                                                       \
            cudaError_t e0_ = cudaSetDevice(c_.device);                             \
            if (e0_ != cudaSuccess) throw Error{DCG_E_CUDA, cudaGetErrorString(e0_)}; \
            body;                                                                   \
        } catch (const Error &e_) {                                                 \
            c_.err = e_.msg;                                                        \
            return e_.code;                                                         \
        } catch (const std::exception &e_) {                                        \
            c_.err = e_.what();                                                     \
            return DCG_E_ARG;                                                       \
        }                                                                           \
    } while (0)

extern "C" {

int dcg_create(int device, int precision, dcg_ctx **out) {
    if (!out) return DCG_E_ARG;
    *out = nullptr;
    if (precision != DCG_PREC_FP64 && precision != DCG_PREC_SPLIT) return DCG_E_ARG;
    dcg_ctx *x = new (std::nothrow) dcg_ctx;
    if (!x) return DCG_E_NOMEM;
    Context &c = x->c;
    c.device = device;
    c.precision = precision;
    try {
        DCG_CUDA(cudaSetDevice(device));
        DCG_CUDA(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking));
        for (int k = 0; k <= dcg::ST_COUNT; k++) DCG_CUDA(cudaEventCreate(&c.ev[k]));
        c.ev_init = true;
        DCG_CUDA(cudaEventCreateWithFlags(&c.aux_fork, cudaEventDisableTiming));
        for (int k = 0; k < Context::kAux; k++) {
            DCG_CUDA(cudaStreamCreateWithFlags(&c.aux[k], cudaStreamNonBlocking));
            DCG_CUDA(cudaEventCreateWithFlags(&c.aux_join[k], cudaEventDisableTiming));
        }
        if (const char *es = getenv("DCG_EIG_STREAMS")) c.eig_streams = std::max(1, std::min(Context::kAux, atoi(es)));
        DCG_CUDA(cudaDeviceGetAttribute(&c.num_sms, cudaDevAttrMultiProcessorCount, device));
        if (const char *ds = getenv("DCG_SPLIT_DESC_STRIDES")) {   // diagnostic: "lbo,sbo"
            int l = 0, s = 0;
            if (sscanf(ds, "%d,%d", &l, &s) == 2 && l > 0 && s > 0 && l % 16 == 0 && s % 16 == 0 && l <= 4096 &&
                s <= 4096) {
                c.split_lbo = l;
                c.split_sbo = s;
            }
        }
        dcg::upload_binomials(c);
        DCG_CUDA(cudaStreamSynchronize(c.stream));
    } catch (const Error &e) {
        int code = e.code;
        dcg_destroy(x);   // releases the streams and events created so far
        return code;
    }
    *out = x;
    return DCG_OK;
}

int dcg_destroy(dcg_ctx *ctx) {
    if (!ctx) return DCG_E_ARG;
    Context &c = ctx->c;
    cudaSetDevice(c.device);
    if (c.stream) cudaStreamSynchronize(c.stream);
    c.ws.release_all();
    delete static_cast<dcg::DevSystem *>(c.dev_state);
    c.dev_state = nullptr;
    if (c.ev_init)
        for (int k = 0; k <= dcg::ST_COUNT; k++) cudaEventDestroy(c.ev[k]);
    for (int k = 0; k < Context::kAux; k++) {
        if (c.aux[k]) {
            cudaStreamSynchronize(c.aux[k]);
            cudaStreamDestroy(c.aux[k]);
        }
        if (c.aux_join[k]) cudaEventDestroy(c.aux_join[k]);
    }
    if (c.aux_fork) cudaEventDestroy(c.aux_fork);
    if (c.stream) cudaStreamDestroy(c.stream);
    delete ctx;
    return DCG_OK;
}

const char *dcg_last_error(const dcg_ctx *ctx) { return ctx ? ctx->c.err.c_str() : "null context"; }

int dcg_set_system(dcg_ctx *ctx, const dcg_system *sys) {
    DCG_API_BODY(ctx, {
        c_.launches = 0;
        for (int k = 0; k < dcg::ST_COUNT; k++) c_.stage_ms[k] = 0.0;
        dcg::set_system(c_, sys);
        return DCG_OK;
    });
}

int dcg_casci(dcg_ctx *ctx, int32_t nroot, double *eigen_out, double *ci_re, double *ci_im, int32_t *ndet_out) {
    DCG_API_BODY(ctx, { return dcg::casci(c_, nroot, eigen_out, ci_re, ci_im, ndet_out); });
}

int dcg_caspt2(dcg_ctx *ctx, uint32_t skip_mask, double e2_sub[8], double sumc2_sub[8], double *e0_out,
               double *etotal_out) {
    if (!e2_sub || !sumc2_sub) return DCG_E_ARG;
    DCG_API_BODY(ctx, { return dcg::caspt2(c_, skip_mask, e2_sub, sumc2_sub, e0_out, etotal_out); });
}

int dcg_caspt2_irreps(const dcg_ctx *ctx, int32_t nsym, double *e2_sym, double *sumc2_sym, int32_t *printed) {
    if (!ctx) return DCG_E_ARG;
    const Context &c = ctx->c;
    if (c.sym_printed.empty()) return DCG_E_STATE;
    if (nsym != c.nsym) return DCG_E_ARG;
    const size_t n = (size_t)8 * c.nsym;
    if (e2_sym) std::copy(c.sym_e2.begin(), c.sym_e2.begin() + n, e2_sym);
    if (sumc2_sym) std::copy(c.sym_sc2.begin(), c.sym_sc2.begin() + n, sumc2_sym);
    if (printed) std::copy(c.sym_printed.begin(), c.sym_printed.begin() + n, printed);
    return DCG_OK;
}

int dcg_casci_determinants(const dcg_ctx *ctx, int64_t *dets_out, int32_t n) {
    if (!ctx || !dets_out) return DCG_E_ARG;
    const Context &c = ctx->c;
    if (!c.have_casci) return DCG_E_STATE;
    if (n < (int32_t)c.dets.size()) return DCG_E_ARG;
    for (size_t i = 0; i < c.dets.size(); i++) dets_out[i] = (int64_t)c.dets[i];
    return DCG_OK;
}

int dcg_get_eps(const dcg_ctx *ctx, double *eps_out, int32_t n) {
    if (!ctx || !eps_out) return DCG_E_ARG;
    const Context &c = ctx->c;
    if ((int)c.eps.size() == 0) return DCG_E_STATE;
    for (int i = 0; i < n && i < (int)c.eps.size(); i++) eps_out[i] = c.eps[i];
    return DCG_OK;
}

int dcg_stage_times(const dcg_ctx *ctx, double *ms_out, int32_t n) {
    if (!ctx || !ms_out) return DCG_E_ARG;
    int k = 0;
    for (; k < n && k < dcg::ST_COUNT; k++) ms_out[k] = ctx->c.stage_ms[k];
    return k;
}

int64_t dcg_kernel_launches(const dcg_ctx *ctx) { return ctx ? ctx->c.launches : -1; }

int dcg_mdcint_canonicalize(dcg_ctx *ctx, const dcg_mdcint_raw *raw, int64_t *nrec_out) {
    if (!raw) return DCG_E_ARG;
    DCG_API_BODY(ctx, {
        c_.mdc_n = dcg::mdcint_canonicalize(c_, *raw, &c_.mdc_ijkl, &c_.mdc_re, &c_.mdc_im);
        c_.mdc_realonly = raw->realonly != 0 || raw->im == nullptr;
        if (nrec_out) *nrec_out = c_.mdc_n;
    });
    return DCG_OK;
}

int dcg_mdcint_records(const dcg_ctx *ctx, int32_t *ijkl_out, double *re_out, double *im_out) {
    if (!ctx || ctx->c.mdc_n < 0) return DCG_E_STATE;
    const Context &c = ctx->c;
    if (cudaSetDevice(c.device) != cudaSuccess) return DCG_E_CUDA;
    const size_t n = (size_t)c.mdc_n;
    if (n == 0) return DCG_OK;
    if ((ijkl_out && cudaMemcpyAsync(ijkl_out, c.mdc_ijkl, 4 * n * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                     c.stream) != cudaSuccess) ||
        (re_out && cudaMemcpyAsync(re_out, c.mdc_re, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream) !=
                       cudaSuccess) ||
        (im_out && cudaMemcpyAsync(im_out, c.mdc_im, n * sizeof(double), cudaMemcpyDeviceToHost, c.stream) !=
                       cudaSuccess) ||
        cudaStreamSynchronize(c.stream) != cudaSuccess)
        return DCG_E_CUDA;
    return DCG_OK;
}

int dcg_set_system_mdcint(dcg_ctx *ctx, const dcg_system *sys, const dcg_mdcint_raw *raw) {
    if (!sys || !raw) return DCG_E_ARG;
    int64_t n = 0;
    int st = dcg_mdcint_canonicalize(ctx, raw, &n);
    if (st != DCG_OK) return st;
    dcg_system s2 = *sys;
    s2.nrec = n;
    s2.rec_ijkl = ctx->c.mdc_ijkl;
    s2.rec_re = ctx->c.mdc_re;
    s2.rec_im = ctx->c.mdc_realonly ? nullptr : ctx->c.mdc_im;
    s2.realonly = ctx->c.mdc_realonly ? 1 : sys->realonly;
    s2.rec_on_device = 1;
    return dcg_set_system(ctx, &s2);
}

int dcg_ivo(dcg_ctx *ctx, int32_t nfsym, const double *mo_energy, int32_t nhomo, double *eps, double *u_re,
            double *u_im, int32_t *block_isym, int32_t *numh_out) {
    DCG_API_BODY(ctx, {
        dcg::ivo(c_, nfsym, mo_energy, nhomo, eps, u_re, u_im, block_isym, numh_out);
        return DCG_OK;
    });
}

int dcg_casci_energy_check(dcg_ctx *ctx, double out[8]) {
    if (!out) return DCG_E_ARG;
    DCG_API_BODY(ctx, {
        dcg::e0test(c_, out);
        return DCG_OK;
    });
}

int dcg_set_merge_reductions(dcg_ctx *ctx, int32_t on) {
    if (!ctx) return DCG_E_ARG;
    ctx->c.merge_reductions = on != 0;
    return DCG_OK;
}

int dcg_merged_reduction_stats(int device, int64_t out[3]) {
    if (!out) return DCG_E_ARG;
    dcg::coop_merge_stats(device, out);
    return DCG_OK;
}

int dcg_set_autotune_trials(dcg_ctx *ctx, int32_t on) {
    if (!ctx) return DCG_E_ARG;
    ctx->c.tune_trials = on != 0;
    return DCG_OK;
}

int dcg_set_casci_solver(dcg_ctx *ctx, int32_t solver) {
    if (!ctx || solver < DCG_CASCI_AUTO || solver > DCG_CASCI_DAVIDSON) return DCG_E_ARG;
    ctx->c.casci_solver = solver;
    return DCG_OK;
}

int32_t dcg_casci_iterations(const dcg_ctx *ctx) { return ctx ? ctx->c.casci_iters : -1; }

int dcg_set_metric_solver(dcg_ctx *ctx, int32_t solver) {
    if (!ctx || solver < DCG_METRIC_AUTO || solver > DCG_METRIC_EIGEN) return DCG_E_ARG;
    ctx->c.metric_solver = solver;
    return DCG_OK;
}

int32_t dcg_gram_cholesky_blocks(const dcg_ctx *ctx) {
    return ctx ? ctx->c.gram_cholesky_blocks + ctx->c.gram_woodbury_blocks : -1;
}

int32_t dcg_gram_deflated_blocks(const dcg_ctx *ctx) { return ctx ? ctx->c.gram_woodbury_blocks : -1; }

int64_t dcg_device_bytes(const dcg_ctx *ctx) { return ctx ? (int64_t)ctx->c.ws.bytes_in_use() : -1; }

int dcg_trim(dcg_ctx *ctx) {
    DCG_API_BODY(ctx, {
        DCG_CUDA(cudaStreamSynchronize(c_.stream));
        c_.ws.release_all();
        delete static_cast<dcg::DevSystem *>(c_.dev_state);
        c_.dev_state = nullptr;
        for (int s = 0; s < Context::kSlots; s++) {
            c_.eig_Q[s] = nullptr;
            c_.eig_n[s] = 0;
            c_.eig_status[s] = nullptr;
        }
        c_.have_system = false;
        c_.have_casci = false;
    });
    return DCG_OK;
}

const char *dcg_version(void) { return "dcaspt2_gb300 0.1 (sm_103a, FP64 path)"; }

void *dcg_stream(const dcg_ctx *ctx) { return ctx ? (void *)ctx->c.stream : nullptr; }

int dcg_zgemm(dcg_ctx *ctx, int precision, int32_t M, int32_t N, int32_t K, int32_t batch, const void *A, int64_t a_si,
              int64_t a_sk, int64_t a_sb, const void *B, int64_t ldb, int32_t conj_b, void *C, int64_t c_si,
              int64_t c_sj, int64_t c_sb, int32_t accumulate) {
    if (M < 0 || N < 0 || K < 0 || batch < 0 || (M * (int64_t)N * batch > 0 && (!A || !B || !C))) return DCG_E_ARG;
    if (precision != DCG_PREC_FP64 && precision != DCG_PREC_SPLIT && precision != DCG_PREC_SPLIT_ACC)
        return DCG_E_ARG;
    DCG_API_BODY(ctx, {
        if ((int64_t)M * N * batch == 0) return DCG_OK;
        const dcg::cplx *a = static_cast<const dcg::cplx *>(A);
        const dcg::cplx *b = static_cast<const dcg::cplx *>(B);
        dcg::cplx *cc = static_cast<dcg::cplx *>(C);
        if (precision == DCG_PREC_SPLIT || precision == DCG_PREC_SPLIT_ACC) {
            dcg::split_reset(c_);
            if (precision == DCG_PREC_SPLIT)
                dcg::zgemm_split(c_, M, N, K, batch, a, a_si, a_sk, a_sb, b, ldb, conj_b ? 1 : 0, cc, c_si, c_sj, c_sb,
                                 accumulate != 0, c_.split_lbo, c_.split_sbo);
            else
                dcg::zgemm_split_acc(c_, M, N, K, batch, a, a_si, a_sk, a_sb, b, ldb, conj_b ? 1 : 0, cc, c_si, c_sj,
                                     c_sb, accumulate != 0);
            if (dcg::split_error(c_)) throw(Error{DCG_E_NUMERIC, "split GEMM: a pipeline wait timed out"});
        } else {
            if (a_si != 1 || c_si != 1) throw(Error{DCG_E_ARG, "FP64 dcg_zgemm needs column-major A and C"});
            const dcg::cplx one = dcg::mk(1.0, 0.0);
            const dcg::cplx beta = accumulate ? one : dcg::mk(0.0, 0.0);
            dcg::zgemm(c_, dcg::OP_N, conj_b ? dcg::OP_R : dcg::OP_N, M, N, K, one, a, a_sk, a_sb, b, ldb, 0, beta, cc,
                       c_sj, c_sb, batch);
        }
        DCG_CUDA(cudaStreamSynchronize(c_.stream));
        return DCG_OK;
    });
}

int dcg_stedc(dcg_ctx *ctx, int32_t n, const double *d, const double *e, double *w_out, double *z_out) {
    if (n < 0 || (n > 0 && (!d || !w_out || (n > 1 && !e)))) return DCG_E_ARG;
    DCG_API_BODY(ctx, {
        if (n == 0) return DCG_OK;
        double *dd = dcg::wsget<double>(c_, "abi.stedc.d", n);
        double *de = dcg::wsget<double>(c_, "abi.stedc.e", n);
        double *w = dcg::wsget<double>(c_, "abi.stedc.w", n);
        DCG_CUDA(cudaMemcpyAsync(dd, d, n * sizeof(double), cudaMemcpyHostToDevice, c_.stream));
        if (n > 1) DCG_CUDA(cudaMemcpyAsync(de, e, (n - 1) * sizeof(double), cudaMemcpyHostToDevice, c_.stream));
        const double *Q = dcg::stedc(c_, n, dd, de, w);
        DCG_CUDA(cudaMemcpyAsync(w_out, w, n * sizeof(double), cudaMemcpyDeviceToHost, c_.stream));
        if (z_out)
            DCG_CUDA(cudaMemcpyAsync(z_out, Q, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost, c_.stream));
        DCG_CUDA(cudaStreamSynchronize(c_.stream));
        return DCG_OK;
    });
}

int dcg_heev_range(dcg_ctx *ctx, int32_t n, const double *a_re, const double *a_im, double *w_out, int32_t vlo,
                   double *z_re, double *z_im) {
    if (n < 0 || vlo < 0 || vlo > n || (n > 0 && (!a_re || !w_out))) return DCG_E_ARG;
    DCG_API_BODY(ctx, {
        if (n == 0) return DCG_OK;
        const size_t nn = (size_t)n * n;
        const size_t nv = (size_t)n * (n - vlo);
        std::vector<dcg::cplx> h(nn);
        for (size_t x = 0; x < nn; x++) h[x] = dcg::mk(a_re[x], a_im ? a_im[x] : 0.0);
        dcg::cplx *A = dcg::wsget<dcg::cplx>(c_, "abi.heev.A", nn);
        dcg::cplx *Z = dcg::wsget<dcg::cplx>(c_, "abi.heev.Z", nv + 1);
        double *w = dcg::wsget<double>(c_, "abi.heev.w", n);
        DCG_CUDA(cudaMemcpyAsync(A, h.data(), nn * sizeof(dcg::cplx), cudaMemcpyHostToDevice, c_.stream));
        dcg::herm_from_upper(c_, n, A, n);
        dcg::heev(c_, n, A, n, w, vlo, z_re ? n : vlo, z_re ? Z : nullptr, n);
        DCG_CUDA(cudaMemcpyAsync(w_out, w, n * sizeof(double), cudaMemcpyDeviceToHost, c_.stream));
        std::vector<dcg::cplx> zh(nv + 1);
        if (z_re && nv) DCG_CUDA(cudaMemcpyAsync(zh.data(), Z, nv * sizeof(dcg::cplx), cudaMemcpyDeviceToHost, c_.stream));
        DCG_CUDA(cudaStreamSynchronize(c_.stream));
        if (z_re)
            for (size_t x = 0; x < nv; x++) {
                z_re[x] = zh[x].x;
                if (z_im) z_im[x] = zh[x].y;
            }
        return DCG_OK;
    });
}

int dcg_heev_batch(dcg_ctx *ctx, int32_t nmat, const int32_t *n, const double *const *a_re,
                   const double *const *a_im, double *const *w_out, double *const *z_re, double *const *z_im) {
    if (nmat < 0 || nmat > dcg::kEigSlots || (nmat > 0 && (!n || !a_re || !w_out))) return DCG_E_ARG;
    for (int q = 0; q < nmat; q++)
        if (n[q] < 0 || (n[q] > 0 && (!a_re[q] || !w_out[q]))) return DCG_E_ARG;
    DCG_API_BODY(ctx, {
        std::vector<dcg::EigJob> jobs;
        std::vector<dcg::cplx *> As;
        std::vector<double *> ws;
        for (int q = 0; q < nmat; q++) {
            const size_t nn = (size_t)n[q] * n[q];
            std::vector<dcg::cplx> h(nn);
            for (size_t x = 0; x < nn; x++) h[x] = dcg::mk(a_re[q][x], (a_im && a_im[q]) ? a_im[q][x] : 0.0);
            dcg::cplx *A = dcg::wsget<dcg::cplx>(c_, "abi.batch.A" + std::to_string(q), nn + 1);
            double *w = dcg::wsget<double>(c_, "abi.batch.w" + std::to_string(q), (size_t)n[q] + 1);
            if (nn) DCG_CUDA(cudaMemcpyAsync(A, h.data(), nn * sizeof(dcg::cplx), cudaMemcpyHostToDevice, c_.stream));
            dcg::herm_from_upper(c_, n[q], A, n[q]);
            dcg::EigJob j;
            j.n = n[q];
            j.A = A;
            j.lda = n[q];
            j.w = w;
            j.slot = q;
            jobs.push_back(j);
            As.push_back(A);
            ws.push_back(w);
        }
        dcg::heev_values_batched(c_, jobs);
        for (int q = 0; q < nmat; q++) {
            const size_t nn = (size_t)n[q] * n[q];
            if (n[q] == 0) continue;
            DCG_CUDA(cudaMemcpyAsync(w_out[q], ws[q], n[q] * sizeof(double), cudaMemcpyDeviceToHost, c_.stream));
            if (z_re && z_re[q]) {
                dcg::cplx *Z = dcg::wsget<dcg::cplx>(c_, "abi.batch.Z", nn);
                dcg::heev_vectors_slot(c_, q, n[q], As[q], n[q], 0, n[q], Z, n[q]);
                std::vector<dcg::cplx> zh(nn);
                DCG_CUDA(cudaMemcpyAsync(zh.data(), Z, nn * sizeof(dcg::cplx), cudaMemcpyDeviceToHost, c_.stream));
                DCG_CUDA(cudaStreamSynchronize(c_.stream));
                for (size_t x = 0; x < nn; x++) {
                    z_re[q][x] = zh[x].x;
                    if (z_im && z_im[q]) z_im[q][x] = zh[x].y;
                }
            }
        }
        DCG_CUDA(cudaStreamSynchronize(c_.stream));
        return DCG_OK;
    });
}

int dcg_heev(dcg_ctx *ctx, int32_t n, const double *a_re, const double *a_im, double *w_out, double *z_re,
             double *z_im) {
    if (n < 0 || (n > 0 && (!a_re || !w_out))) return DCG_E_ARG;
    DCG_API_BODY(ctx, {
        if (n == 0) return DCG_OK;
        const size_t nn = (size_t)n * n;
        std::vector<dcg::cplx> h(nn);
        for (size_t x = 0; x < nn; x++) h[x] = dcg::mk(a_re[x], a_im ? a_im[x] : 0.0);
        dcg::cplx *A = dcg::wsget<dcg::cplx>(c_, "abi.heev.A", nn);
        dcg::cplx *Z = dcg::wsget<dcg::cplx>(c_, "abi.heev.Z", nn);
        double *w = dcg::wsget<double>(c_, "abi.heev.w", n);
        DCG_CUDA(cudaMemcpyAsync(A, h.data(), nn * sizeof(dcg::cplx), cudaMemcpyHostToDevice, c_.stream));
        dcg::herm_from_upper(c_, n, A, n);
        dcg::heev(c_, n, A, n, w, 0, z_re ? n : 0, z_re ? Z : nullptr, n);
        DCG_CUDA(cudaMemcpyAsync(w_out, w, n * sizeof(double), cudaMemcpyDeviceToHost, c_.stream));
        if (z_re) DCG_CUDA(cudaMemcpyAsync(h.data(), Z, nn * sizeof(dcg::cplx), cudaMemcpyDeviceToHost, c_.stream));
        DCG_CUDA(cudaStreamSynchronize(c_.stream));
        if (z_re)
            for (size_t x = 0; x < nn; x++) {
                z_re[x] = h[x].x;
                if (z_im) z_im[x] = h[x].y;
            }
        return DCG_OK;
    });
}

int dcg_solve_h(dcg_ctx *ctx, const void *hclass, int32_t ninact, int32_t nsec, const double *eps_i,
                const double *eps_s, const int32_t *irp_i, const int32_t *irp_s, const int32_t *multb_d,
                const int32_t *multb_s, int32_t nsymrpa, double eshift, double out[2]) {
    if (!out || ninact < 0 || nsec < 0 || nsymrpa < 1) return DCG_E_ARG;
    if ((int64_t)ninact * nsec > 0 && (!hclass || !eps_i || !eps_s || !irp_i || !irp_s || !multb_d || !multb_s))
        return DCG_E_ARG;
    DCG_API_BODY(ctx, {
        out[0] = out[1] = 0.0;
        if ((int64_t)ninact * nsec == 0) return DCG_OK;
        const int nblk = dcg::h_stream_blocks(ninact, nsec);
        double *part = dcg::wsget<double>(c_, "hsolve.part", 2 * (size_t)nblk);
        double *red = dcg::wsget<double>(c_, "hsolve.red", 2);
        dcg::launch_h_stream2(c_, static_cast<const dcg::cplx *>(hclass), ninact, nsec, eps_i, eps_s, irp_i, irp_s,
                              multb_d, multb_s, nsymrpa, eshift, part, part + nblk);
        dcg::dsum(c_, part, nblk, red);
        dcg::dsum(c_, part + nblk, nblk, red + 1);
        DCG_CUDA(cudaMemcpyAsync(out, red, 2 * sizeof(double), cudaMemcpyDeviceToHost, c_.stream));
        DCG_CUDA(cudaStreamSynchronize(c_.stream));
        return DCG_OK;
    });
}

int dcg_set_wait_limit(dcg_ctx *ctx, double seconds) {
    if (!ctx || !(seconds >= 0.0) || seconds > 60.0) return DCG_E_ARG;
    // 0 restores the defaults; any positive limit is at least 1 ns
    ctx->c.wait_limit_ns = seconds == 0.0 ? 0 : std::max<uint64_t>(1, (uint64_t)(seconds * 1.0e9));
    return DCG_OK;
}

int dcg_time_family(dcg_ctx *ctx, int32_t family) {
    if (!ctx || family < 0 || family > DCG_FAM_SPLIT_MMA) return DCG_E_ARG;
    Context &c = ctx->c;
    dcg::fam_collect(c);
    c.fam = family;
    c.fam_ms = 0.0;
    c.fam_work = 0.0;
    c.fam_launches = 0;
    return DCG_OK;
}

int dcg_family_stats(const dcg_ctx *ctx, double *ms, int64_t *launches, double *work) {
    if (!ctx) return DCG_E_ARG;
    const Context &c = ctx->c;
    // fold in events still pending from calls that do not collect them (dcg_heev, dcg_stedc)
    cudaSetDevice(c.device);
    dcg::fam_collect(const_cast<Context &>(c));
    if (ms) *ms = c.fam_ms;
    if (launches) *launches = c.fam_launches;
    if (work) *work = c.fam_work;
    return DCG_OK;
}

}  // extern "C"
