// Shared definitions of the GB300 CASCI/CASPT2 library: complex helpers, the context,
// workspace management and launch accounting.  Host code is C++17; device code targets
// sm_103a only.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <cstdlib>
#include <map>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/dcaspt2_gb300.h"

namespace dcg {

typedef double2 cplx;

// ---------------------------------------------------------------- complex arithmetic
__host__ __device__ __forceinline__ cplx mk(double r, double i) { return make_double2(r, i); }
__host__ __device__ __forceinline__ cplx cadd(cplx a, cplx b) { return mk(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ cplx csub(cplx a, cplx b) { return mk(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ cplx cmul(cplx a, cplx b) {
    return mk(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__host__ __device__ __forceinline__ cplx cconj(cplx a) { return mk(a.x, -a.y); }
__host__ __device__ __forceinline__ cplx cscale(cplx a, double s) { return mk(a.x * s, a.y * s); }
__host__ __device__ __forceinline__ double cabs2(cplx a) { return a.x * a.x + a.y * a.y; }
// a*conj(b)
__host__ __device__ __forceinline__ cplx cmulc(cplx a, cplx b) {
    return mk(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y);
}
// acc += a*b
__host__ __device__ __forceinline__ void cfma(cplx &acc, cplx a, cplx b) {
    acc.x = fma(a.x, b.x, acc.x);
    acc.x = fma(-a.y, b.y, acc.x);
    acc.y = fma(a.x, b.y, acc.y);
    acc.y = fma(a.y, b.x, acc.y);
}
__host__ __device__ __forceinline__ cplx cdiv(cplx a, cplx b) {
    double d = b.x * b.x + b.y * b.y;
    return mk((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// ---------------------------------------------------------------- status / errors
struct Error {
    int code;
    std::string msg;
};

// ---------------------------------------------------------------- context
struct Context;

// Grow-only named device workspace: buffers survive across solves so a served or
// benchmarked loop allocates once.
class Workspace {
  public:
    void *get(const std::string &name, size_t bytes);
    // page-locked host buffer (small per-step readbacks), kept like the device buffers
    void *host(const std::string &name, size_t bytes);
    void release_all();
    size_t bytes_in_use() const { return total_; }
    ~Workspace() { release_all(); }

  private:
    struct Buf {
        void *p = nullptr;
        size_t bytes = 0;
    };
    std::map<std::string, Buf> bufs_, host_;
    size_t total_ = 0;
};

// Stage indices of dcg_stage_times
enum Stage {
    ST_INTS = 0, ST_CASMAT, ST_CASEIG, ST_FOCK, ST_CIROT, ST_RDM, ST_TRANS,
    ST_A, ST_B, ST_C, ST_D, ST_E, ST_F, ST_G, ST_H, ST_AC, ST_BDEFG, ST_COUNT
};

struct Context {
    int device = 0;
    int precision = DCG_PREC_FP64;
    cudaStream_t stream = nullptr;
    // auxiliary streams for independent eigensolver jobs, forked from and joined back to
    // `stream` (DCG_EIG_STREAMS: how many are used, 1 = none)
    static constexpr int kAux = 4;
    cudaStream_t aux[kAux] = {};
    cudaEvent_t aux_fork = nullptr, aux_join[kAux] = {};
    int eig_streams = kAux;
    Workspace ws;
    std::string err;
    int64_t launches = 0;
    int num_sms = 0;
    // limit of the device-side waits that can give up (grid barriers of the tridiagonalisation,
    // pipeline waits of the tensor-core GEMM), ns; 0 = each kernel's default (dcg_set_wait_limit)
    uint64_t wait_limit_ns = 0;
    bool tune_trials = true;     // may run autotuner trials (off for serving slots)
    // hand batched tridiagonal reductions to the device's batcher, which merges those of all
    // contexts that set it into joint cooperative launches (on for serving slots)
    bool merge_reductions = false;
    void *dev_state = nullptr;   // device-side system state (owned, see dcg_api.cu)

    // ---- per-family kernel timing (dcg_time_family)
    int fam = 0;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> fam_ev;
    double fam_ms = 0.0, fam_work = 0.0;
    // tcgen05 shared-memory descriptor strides of the split GEMM (leading, stride byte offset)
    int split_lbo = 128, split_sbo = 256;
    // per eigensolver slot: tridiagonal eigenvectors of the last value stage (device, n x n),
    // their dimension and the divide-and-conquer status word
    static constexpr int kSlots = 32;
    const double *eig_Q[kSlots] = {};
    int eig_n[kSlots] = {};
    int *eig_status[kSlots] = {};
    int64_t fam_launches = 0;
    // CASCI eigensolver: DCG_CASCI_AUTO, _DENSE or _DAVIDSON (dcg_set_casci_solver)
    int casci_solver = 0;
    int casci_iters = 0;   // Davidson iterations of the last CASCI (0: dense solver)
    // Gram-route metric: DCG_METRIC_AUTO (Cholesky solve when K - 1e-8 I is positive
    // definite, else eigendecomposition) or DCG_METRIC_EIGEN (dcg_set_metric_solver)
    int metric_solver = 0;
    int gram_cholesky_blocks = 0;   // Gram blocks of the last dcg_caspt2 solved by Cholesky
    int gram_woodbury_blocks = 0;   // ... of them with metric eigenvalues under the cutoff deflated
    // per-irrep results of the last dcg_caspt2, [sub * nsym + isym - 1] for subspaces A..H:
    // e2X(isym), its c^2 share, and whether solve_X_subspace prints the e2X(isym) line
    // (a symmetry block with dimn > 0 whose S keeps dimm > 0 vectors above the cutoff)
    std::vector<double> sym_e2, sym_sc2;
    std::vector<int32_t> sym_printed;
    // last MDCINT canonicalisation (device, in the workspace)
    int64_t mdc_n = -1;
    int32_t *mdc_ijkl = nullptr;
    double *mdc_re = nullptr, *mdc_im = nullptr;
    bool mdc_realonly = false;

    // ---- system (host copies)
    bool have_system = false;
    int ni = 0, na = 0, ns = 0, ne = 0, nmo = 0, nsym = 1, totsym = 1, selectroot = 1;
    bool realonly = false;
    double eshift = 0.0, ecore = 0.0;
    std::vector<int> multb;   // 2n x 2n column-major
    std::vector<int> irpamo;  // nmo
    std::vector<cplx> h;      // nmo x nmo column-major
    int ras1 = 0, ras2 = 0, ras3 = 0, ras1_max_hole = 0, ras3_max_elec = 0;
    int min_hole_ras1 = 0, min_elec_ras3 = 0;
    int64_t nrec = 0;

    // ---- CASCI results
    bool have_casci = false;
    std::vector<uint64_t> dets;        // CI space, Gosper order
    std::vector<double> ecas;          // eigenvalues (+ ecore) of the computed roots
    int nroot_done = 0;
    std::vector<double> eps;           // after fockdiag

    // ---- timings
    cudaEvent_t ev[ST_COUNT + 1];
    bool ev_init = false;
    double stage_ms[ST_COUNT] = {0};

    // multiplication tables (read_mrconee.F90:368-453), 1-based values, [a-1][b-1]
    std::vector<int> multb_s, multb_d, multb_ds;

    int md(int a, int b) const { return multb_d[(a - 1) * nsym + (b - 1)]; }
    int ms(int a, int b) const { return multb_s[(a - 1) * nsym + (b - 1)]; }
};

// ---------------------------------------------------------------- helpers
#define DCG_CUDA(call)                                                                  \
    do {                                                                                \
        cudaError_t e_ = (call);                                                        \
        if (e_ != cudaSuccess)                                                          \
            throw ::dcg::Error{DCG_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)}; \
    } while (0)

#define DCG_LAUNCHED(ctx)                                                               \
    do {                                                                                \
        (ctx).launches++;                                                               \
        cudaError_t e_ = cudaGetLastError();                                            \
        if (e_ != cudaSuccess)                                                          \
            throw ::dcg::Error{DCG_E_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e_)}; \
    } while (0)

inline unsigned grid1d(int64_t n, int block) { return (unsigned)((n + block - 1) / block); }

template <typename T>
T *wsget(Context &c, const std::string &name, size_t count) {
    return reinterpret_cast<T *>(c.ws.get(name, count * sizeof(T) + 256));
}

// A host vector copied into the named workspace buffer (stream-ordered).
template <typename T>
T *upload(Context &c, const std::string &name, const std::vector<T> &v) {
    T *p = wsget<T>(c, name, v.size() + 1);
    if (!v.empty()) DCG_CUDA(cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c.stream));
    return p;
}

// n elements of device memory read back (synchronises the context's stream).
template <typename T>
std::vector<T> download(Context &c, const T *p, size_t n) {
    std::vector<T> v(n);
    if (n) DCG_CUDA(cudaMemcpyAsync(v.data(), p, n * sizeof(T), cudaMemcpyDeviceToHost, c.stream));
    DCG_CUDA(cudaStreamSynchronize(c.stream));
    return v;
}

// ---------------------------------------------------------------- autotuner
// A process-wide table of tuned choices, keyed by the decision and the problem shape.  The
// first call of a key with trial_ok runs every candidate once (untimed, so workspaces grow
// outside the timing), then times each on the caller's stream with CUDA events (best of two)
// and keeps the fastest; later calls of the key, in any context, reuse it.  Candidate 0 is the
// built-in heuristic, used while tuning is off (dcg_autotune_mode) and for keys first met
// without trial_ok.  The trial runs must leave the same result as the final run.
enum TuneKind { TUNE_ZGEMM = 1, TUNE_SPLIT_KERNEL = 2 };
struct TuneKey {
    int kind, ops, m, n, k, flags;
    bool operator<(const TuneKey &o) const {
        if (kind != o.kind) return kind < o.kind;
        if (ops != o.ops) return ops < o.ops;
        if (m != o.m) return m < o.m;
        if (n != o.n) return n < o.n;
        if (k != o.k) return k < o.k;
        return flags < o.flags;
    }
};
int autotune_run(Context &c, const TuneKey &key, int ncand, bool trial_ok, void (*fn)(void *, int), void *arg);
template <typename F>
int autotune(Context &c, const TuneKey &key, int ncand, bool trial_ok, F &&run) {
    using Fn = typename std::remove_reference<F>::type;
    return autotune_run(c, key, ncand, trial_ok, [](void *p, int q) { (*static_cast<Fn *>(p))(q); },
                        const_cast<void *>(static_cast<const void *>(&run)));
}

// Diagnostic: with DCG_GEMM_TRACE=1 in the environment, each GEMM call is timed by CUDA events
// (synchronising the stream) and printed to stderr as "gemm <kind> m n k batch <ms>".
struct GemmTrace {
    Context &c;
    const char *kind;
    int m, n, k, batch;
    cudaEvent_t a = nullptr, b = nullptr;
    static bool enabled() {
        static const bool on = [] {
            const char *e = getenv("DCG_GEMM_TRACE");
            return e && e[0] == '1';
        }();
        return on;
    }
    GemmTrace(Context &c_, const char *kind_, int m_, int n_, int k_, int batch_)
        : c(c_), kind(kind_), m(m_), n(n_), k(k_), batch(batch_) {
        if (!enabled()) return;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, c.stream);
    }
    ~GemmTrace() {
        if (!a) return;
        cudaEventRecord(b, c.stream);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        fprintf(stderr, "gemm %s %d %d %d %d %.4f\n", kind, m, n, k, batch, ms);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
    }
};

// Records CUDA events around the launches of one kernel family when that family is
// selected; elapsed times are collected by fam_collect() after the stream synchronises.
struct FamScope {
    Context &c;
    bool on;
    int64_t l0;
    cudaEvent_t a = nullptr, b = nullptr;
    FamScope(Context &cc, int family, double work) : c(cc), on(cc.fam == family && family != 0), l0(cc.launches) {
        if (!on) return;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, c.stream);
        c.fam_work += work;
    }
    ~FamScope() {
        if (!on) return;
        cudaEventRecord(b, c.stream);
        c.fam_ev.push_back({a, b});
        c.fam_launches += c.launches - l0;
    }
};
void fam_collect(Context &c);

// Runs f(k) for k in [0, njob), job k's launches on auxiliary stream k mod (streams used):
// the streams first wait for the context stream, and the context stream waits for all of them
// after, so the jobs overlap each other and nothing else.  The jobs must share no buffers.
template <class F>
void on_aux_streams(Context &c, int njob, F &&f) {
    const int used = std::min(std::min(c.eig_streams, (int)Context::kAux), njob);
    if (used <= 1) {
        for (int k = 0; k < njob; k++) f(k);
        return;
    }
    cudaStream_t main = c.stream;
    DCG_CUDA(cudaEventRecord(c.aux_fork, main));
    for (int s = 0; s < used; s++) DCG_CUDA(cudaStreamWaitEvent(c.aux[s], c.aux_fork, 0));
    auto join = [&]() {
        c.stream = main;
        for (int s = 0; s < used; s++) {
            cudaEventRecord(c.aux_join[s], c.aux[s]);
            cudaStreamWaitEvent(main, c.aux_join[s], 0);
        }
    };
    try {
        for (int k = 0; k < njob; k++) {
            c.stream = c.aux[k % used];
            f(k);
        }
    } catch (...) {
        join();
        throw;
    }
    join();
}

// ---------------------------------------------------------------- linear algebra (dcg_linalg.cu)
enum Op { OP_N = 0, OP_T = 1, OP_C = 2, OP_R = 3 };   // R = conjugate without transpose

// C = alpha*op(A)*op(B) + beta*C, column-major, batched with element strides.
void zgemm(Context &c, Op opa, Op opb, int m, int n, int k, cplx alpha, const cplx *A, int64_t lda,
           int64_t sa, const cplx *B, int64_t ldb, int64_t sb, cplx beta, cplx *C, int64_t ldc,
           int64_t sc, int batch = 1);

// Hermitian eigendecomposition of A (n x n, lda), ascending eigenvalues in w (device).
// Eigenvectors for eigenvalue indices [vlo, n) are written to Z (n x (n-vlo), ldz) as
// columns 0..n-vlo-1.  A is destroyed.  Pass vlo = n for eigenvalues only.
void heev(Context &c, int n, cplx *A, int64_t lda, double *w, int vlo, int vhi, cplx *Z, int64_t ldz);

// Batched Hermitian eigensolver: job = one matrix (A, n x n, lda; destroyed), its eigenvalues
// w (device, ascending) and a workspace slot (0 .. kEigSlots-1, distinct within a batch; slot 0
// is the one heev() uses).
constexpr int kEigSlots = Context::kSlots;
struct EigJob {
    int n = 0;
    cplx *A = nullptr;
    int64_t lda = 0;
    double *w = nullptr;
    int slot = 0;
    bool tridiag_only = false;   // stop after the reduction: for tridiag_e2 (w is not written)
};
void heev_values_batched(Context &c, const std::vector<EigJob> &jobs);
void heev_vectors_slot(Context &c, int slot, int n, cplx *A, int64_t lda, int vlo, int vhi, cplx *Z, int64_t ldz);

// Eigenvectors [vlo, vhi) of the matrix most recently passed to heev() (same A, w).
void heev_vectors_only(Context &c, int n, cplx *A, int64_t lda, const double *w, int vlo, int vhi, cplx *Z,
                       int64_t ldz);

// Split-precision (BF16 tensor core, FP64 recombination) complex GEMM, dcg_split.cu:
// C[z*c_sb + i*c_si + j*c_sj] (+)= sum_k A[z*a_sb + i*a_si + k*a_sk] * op(B)(k, j),
// op(B)(k, j) = B[k + j*ldb] (conj_b 0) or its conjugate (conj_b 1).
void zgemm_split(Context &c, int M, int N, int K, int batch, const cplx *A, int64_t a_si, int64_t a_sk, int64_t a_sb,
                 const cplx *B, int64_t ldb, int opb, cplx *C, int64_t c_si, int64_t c_sj, int64_t c_sb,
                 bool accumulate, int lbo, int sbo);
// The same product through the seven-slice kernel (~2^-45 instead of ~2^-36 relative per term),
// for contractions whose errors the metric's inverse amplifies.
void zgemm_split_acc(Context &c, int M, int N, int K, int batch, const cplx *A, int64_t a_si, int64_t a_sk,
                     int64_t a_sb, const cplx *B, int64_t ldb, int opb, cplx *C, int64_t c_si, int64_t c_sj,
                     int64_t c_sb, bool accumulate);
void split_reset(Context &c);
int split_error(Context &c);

// Symmetric tridiagonal eigendecomposition by divide and conquer (d: n, e: n-1, device);
// ascending eigenvalues into w, eigenvectors returned (n x n, ld n, workspace-owned).
const double *stedc(Context &c, int n, const double *d, const double *e, double *w);

// Largest B' dimension that tridiag_e2 takes (the reflections hold a column in registers).
constexpr int kTridiagE2MaxN = 1024;
// E2 terms of a B' matrix reduced to tridiagonal form T (B' = Q T Q^H) in `slot` by a
// tridiag_only job, without its eigendecomposition: with y_o = Q^H VC[:, o] (VC: n x nouter),
//   e2o[o] = -Re y_o^H (T + alpha_o)^-1 y_o,   sco[o] = |(T + alpha_o)^-1 y_o|^2,
// which equal the reference's -sum_m |W^H v|_m^2 / (alpha + w_m) and sum_m |W^H v|_m^2 /
// (alpha + w_m)^2 over the eigenpairs (w_m, W) of B'.  n <= kTridiagE2MaxN.
void tridiag_e2(Context &c, int slot, int n, const cplx *A, int64_t lda, const cplx *VC, int64_t ldvc, int nouter,
                const double *alpha, double *e2o, double *sco);

// The same E2 terms from a band form: B' (n x n, both triangles, destroyed) reduced to a Hermitian
// matrix of lower bandwidth kBandNB by blocked Householder panels (FP64 GEMM trailing updates),
// y_o = Q^H VC[:, o], then one banded solve with partial pivoting per outer index (dcg_band.cu).
// band_e2_pays: whether B' of dimension n with nouter outer indices takes it: only when the
// environment variable DCG_BPRIME_ROUTE = band asks for it (measured slower than the
// tridiagonal form on GB300, see dcg_band.cu; kBandMinN is the size it was measured from).
constexpr int kBandNB = 16;
constexpr int kBandMinN = 256;
bool band_e2_pays(int n, int nouter);
void band_e2(Context &c, int slot, int n, cplx *A, int64_t lda, const cplx *VC, int64_t ldvc, int nouter,
             const double *alpha, double *e2o, double *sco);

// heev_vectors_slot and tridiag_e2 calls of distinct slots, overlapped on the auxiliary
// streams (vector jobs above 1024 rows share the blocked back-transformation's workspace and
// run first, on the context stream).  The family timers see the overlapped group once.
struct VecJob {
    int slot = 0, n = 0;
    cplx *A = nullptr;
    int64_t lda = 0;
    int vlo = 0, vhi = 0;
    cplx *Z = nullptr;
    int64_t ldz = 0;
};
struct TE2Job {
    int slot = 0, n = 0;
    const cplx *A = nullptr;
    int64_t lda = 0;
    const cplx *VC = nullptr;
    int64_t ldvc = 0;
    int nouter = 0;
    const double *alpha = nullptr;
    double *e2o = nullptr, *sco = nullptr;
};
void eig_slot_jobs(Context &c, const std::vector<VecJob> &vj, const std::vector<TE2Job> &tj);

// Solve A x = b (n x n, LU with partial pivoting), b overwritten.  Returns info.
int zgesv(Context &c, int n, cplx *A, int64_t lda, cplx *b);

// Upper triangle of C = A A^H (n x n from A n x k); the strictly lower part is left undefined.
void zherk_upper(Context &c, int n, int k, const cplx *A, int64_t lda, cplx *C, int64_t ldc);

// Hermitian fill from the upper triangle (ZHEEV uplo='U' semantics): A(j,i) = conj(A(i,j))
// for i < j, Im A(i,i) = 0.
void herm_from_upper(Context &c, int n, cplx *A, int64_t lda);

// Joint-launch counters of the merged tridiagonal reductions on a device (dcg_eig.cu): launches,
// launches that carried more than one context's submission, submissions carried.
void coop_merge_stats(int device, int64_t out[3]);

// deterministic sum of n doubles on the device into *out (device)
void dsum(Context &c, const double *x, int64_t n, double *out);

// Cholesky A = L L^H of a Hermitian matrix (lower triangle, in place; dcg_chol.cu); *info
// (device) = index + 1 of the first non-positive pivot, 0 when A is positive definite.
void zpotrf_lower(Context &c, int n, cplx *A, int64_t lda, int *info);
// A X = B with the factor of zpotrf_lower; B (n x nrhs, ldb) overwritten by X.
void zpotrs_lower(Context &c, int n, const cplx *L, int64_t lda, cplx *B, int64_t ldb, int nrhs);
// Per outer index o: e2o = -Re u^H z, sco = |z|^2, z the solution on the orthogonal complement
// of the r columns of Ps (Mp x r, orthonormal) of the compression of D + alpha_o (D diagonal),
// u = U[:, o] in that complement (dcg_chol.cu).
void launch_woodbury_e2(Context &c, int Mp, int r, const cplx *U, int64_t ldu, const cplx *Ps, int64_t ldp,
                        const double *Dd, const double *alpha, int nouter, double *e2o, double *sco);

// MDCINT -> MDCINTNEW on the device (dcg_mdcint.cu); returns the record count, the stream
// (workspace buffers) through the pointers.
int64_t mdcint_canonicalize(Context &c, const dcg_mdcint_raw &raw, int32_t **ijkl_out, double **re_out,
                            double **im_out);

// Sparse CASCI Hamiltonian (CSR, rows in CI order, diagonal first in each row).
struct CsrMatrix {
    int n = 0;
    int64_t nnz = 0;
    int64_t *rowptr = nullptr;
    int *cols = nullptr;
    cplx *vals = nullptr;
    double *diag = nullptr;
};
// The Slater-Condon elements of the CI space as CSR (dcg_ci.cu).
void build_casmat_csr(Context &c, const uint64_t *dets, int ndet, const cplx *h, const cplx *g, CsrMatrix &m);
// Lowest nwant eigenpairs of the CSR Hamiltonian by block Davidson (dcg_davidson.cu):
// eigenvalues to w (device), vectors to Z (n x nwant); |r| <= tol_rel max(1, max|H_ii|).
void davidson_lowest_csr(Context &c, const CsrMatrix &H, int nwant, double *w, cplx *Z, double tol_rel, int maxit);

// IVO (dcg_ivo.cu): the Fock matrix of the secondary spinors from (ab|kk) and (ak|kb) over the
// active HOMO spinors [k0, k1), e_sec the secondary orbital energies (host), and the
// eigenpairs of each block of secondary indices by the LAPACK ZHEEV algorithm.
void ivo_blocks_eig(Context &c, const cplx *F1A, const cplx *F2A, const double *e_sec_host, int k0, int k1, int odd,
                    double numh, const std::vector<std::vector<int>> &blocks, std::vector<std::vector<double>> &w_out,
                    std::vector<std::vector<cplx>> &v_out);


}  // namespace dcg
