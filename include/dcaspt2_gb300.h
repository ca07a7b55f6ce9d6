/*
 * dcaspt2_gb300.h -- C ABI of the GB300 CASCI/CASPT2 hot path.
 *
 * The reference program (DIRAC-CASPT2, Fortran) reaches this path through two
 * argument-less driver calls that communicate through module globals and scratch
 * files:
 *   r4dcasci       (src/r4dcasci.F90:1-134, called from src/dcaspt2_run_subprograms.F90:57)
 *   r4dcaspt2_tra  (src/r4dcaspt2_tra.F90:4-482, called from src/dcaspt2_run_subprograms.F90:62)
 * The Fortran side keeps its input parser and MRCONEE/MDCINT readers
 * (read_input, read_mrconee, check_realonly, create_newmdcint) and hands the results
 * to this library; everything from readint2_casci onwards runs on the GPU.
 *
 * Conventions
 *   - every entry point returns an int status: 0 = success, negative = library error
 *     (DCG_E_*), positive = LAPACK-style info of a failed factorisation;
 *     dcg_last_error() gives a one-line message.  The library never exits the process.
 *   - arrays are column-major (Fortran order); spinor indices are 1-based CAS order
 *     (inactive, active, secondary, sorted by orbital energy) as produced by
 *     read_mrconee; complex values are passed as separate real and imaginary planes,
 *     the storage of the reference (one_elec_int_r/_i, cir/cii).
 *   - the caller owns all host arrays; they are read during the call only.
 *   - one context per host thread; a context owns one CUDA stream on one device.
 */
#ifndef DCASPT2_GB300_H
#define DCASPT2_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DCG_OK 0
#define DCG_E_ARG (-1)        /* invalid argument / inconsistent dimensions            */
#define DCG_E_CUDA (-2)       /* CUDA runtime error (message in dcg_last_error)         */
#define DCG_E_STATE (-3)      /* call order violated (e.g. caspt2 before casci)         */
#define DCG_E_NODET (-4)      /* no CASCI configuration for totsym (search_cas_configuration.F90:158-172) */
#define DCG_E_NOMEM (-5)      /* device memory exhausted                                */
#define DCG_E_NUMERIC (-6)    /* eigensolver or solver did not converge                 */
#define DCG_E_IO (-7)         /* file missing, truncated or not in the expected format  */

/* precision of the dense contractions (the transformation and S/B/V builds) */
#define DCG_PREC_FP64 0       /* native FP64 everywhere                                  */
#define DCG_PREC_SPLIT 1      /* split-precision tensor-core contractions, FP64 recombine */
#define DCG_PREC_SPLIT_ACC 2  /* dcg_zgemm only: the seven-slice split product (~2^-45 relative per
                                 term instead of ~2^-36), which the split path uses for the Gram
                                 metric and the products Lambda^-1 amplifies                  */

typedef struct dcg_ctx dcg_ctx;

/* The system one CASCI/CASPT2 solve consumes: the module globals the reference's
 * readers fill (src/module_global_variables.F90) plus the MDCINTNEW record stream
 * (src/create_newmdcint.F90:171-177). */
typedef struct dcg_system {
    int32_t ninact, nact, nsec, nelec;   /* .ninact .nact .nsec .nelec                     */
    int32_t nmo;                         /* NMO of MRCONEE (may exceed ninact+nact+nsec)   */
    int32_t nsymrpa;                     /* abelian double-group irreps; MULTB is 2n x 2n  */
    int32_t totsym, selectroot;          /* .caspt2_ciroots entry                          */
    int32_t realonly;                    /* MDCINT realonly (module_realonly.F90:29-77)    */
    double eshift;                       /* .eshift                                        */
    double ecore;                        /* ECORE of MRCONEE                               */
    const int32_t *multb;                /* MULTB(2n,2n), 1-based values                   */
    const int32_t *irpamo;               /* irpamo(nmo), CAS order, 1-based                */
    const double *h_re, *h_im;           /* one_elec_int_r/_i (nmo,nmo), CAS order         */
    int64_t nrec;                        /* number of MDCINTNEW records                    */
    const int32_t *rec_ijkl;             /* (4,nrec): i,j,k,l of (ij|kl), 1-based CAS      */
    const double *rec_re, *rec_im;       /* values; rec_im may be NULL when realonly       */
    int32_t ras1_size, ras2_size, ras3_size;          /* RAS partition sizes (0 = CAS)      */
    int32_t ras1_max_hole, ras3_max_elec;             /* .ras1 / .ras3 limits               */
    int32_t min_hole_ras1, min_elec_ras3;             /* .minholeras1 / .minelecras3        */
    int32_t rec_on_device;               /* 1: rec_ijkl/rec_re/rec_im are device pointers on the
                                            context's device (already resident in HBM)           */
} dcg_system;

/* DIRAC's MDCINT file(s) as read record by record (MDCINT, MDCINXXXX1, ...: header
 * `datex, timex, nkr, (kr(i), kr(-i), i = 1..nkr)`, then records `ikr, jkr, nz, (indk, indl),
 * values`; read_mrconee.F90 / create_newmdcint.F90:3-171), flattened: the caller's input to
 * dcg_mdcint_canonicalize / dcg_set_system_mdcint, which replace create_newmdcint. */
typedef struct dcg_mdcint_raw {
    int64_t nrec;                        /* records (ikr, jkr) over all files, in file order   */
    int64_t nent;                        /* entries (sum of nz)                                 */
    const int64_t *rec_off;              /* nrec + 1: entries of record r are rec_off[r] ..     */
    const int32_t *ikr, *jkr;            /* per record, signed Kramers-pair indices             */
    const int32_t *indk, *indl;          /* per entry, signed                                   */
    const double *re, *im;               /* per entry, as stored; im NULL when real-only        */
    int32_t nkr;                         /* header: number of Kramers pairs                     */
    const int32_t *kr;                   /* header: (kr(i), kr(-i)) for i = 1..nkr, 2 x nkr     */
    int32_t nmo;                         /* MRCONEE NMO                                          */
    const int32_t *dirac_to_cas;         /* nmo + 1 (entry 0 unused): DIRAC spinor -> CAS index */
    int32_t scheme;                      /* .mdcint_scheme of the input (6: both orders stored) */
    int32_t realonly;                    /* MDCINT real-only (module_realonly.F90:29-77)         */
} dcg_mdcint_raw;

/* Create a context on CUDA device `device`.  precision: DCG_PREC_*. */
int dcg_create(int device, int precision, dcg_ctx **out);
int dcg_destroy(dcg_ctx *ctx);
const char *dcg_last_error(const dcg_ctx *ctx);

/* Upload a system and expand its integrals on the device (replaces readint2_casci,
 * src/module_2integrals.F90:26-588, and divide_2_elec_integral_into_subspaces,
 * src/divide_2_elec_integral_into_subspaces.F90:3-409). */
int dcg_set_system(dcg_ctx *ctx, const dcg_system *sys);

/* The MDCINTNEW record stream of create_newmdcint (create_newmdcint.F90:3-321) built on the
 * device from the raw MDCINT records: both Kramers partners of every record, bra/ket-exchanged
 * copies for schemes other than 6, the TYPE1-4 canonical filter, the 0.25e-12 cutoff, CAS
 * order, in the reference's output order.  The stream stays in the context (device); *nrec_out
 * receives its length. */
int dcg_mdcint_canonicalize(dcg_ctx *ctx, const dcg_mdcint_raw *raw, int64_t *nrec_out);
/* Copy the last canonicalised stream to host arrays: ijkl_out (4 x nrec, 1-based CAS indices
 * (i, j, k, l) of (ij|kl)), re_out and im_out (nrec; im_out may be NULL). */
int dcg_mdcint_records(const dcg_ctx *ctx, int32_t *ijkl_out, double *re_out, double *im_out);
/* dcg_mdcint_canonicalize then dcg_set_system on the device-resident stream (the record fields
 * of sys are ignored): MDCINT to expanded integrals without a scratch file or a host copy of
 * MDCINTNEW. */
int dcg_set_system_mdcint(dcg_ctx *ctx, const dcg_system *sys, const dcg_mdcint_raw *raw);

/* CASCI (replaces casci, src/casci.F90:3-163: search_cas_configuration, casmat,
 * cdiag/rdiag).  Writes min(nroot, ndet) total energies eigen(i) = ecas(i) + ecore
 * and, when ci_re is not NULL, the CI coefficients cir/cii (ndet, nroot) that the
 * reference stores in CIDATA_sym<n>.  *ndet_out receives ndet. */
int dcg_casci(dcg_ctx *ctx, int32_t nroot, double *eigen_out, double *ci_re, double *ci_im,
              int32_t *ndet_out);

/* CASPT2 for ctx->selectroot (replaces r4dcaspt2_tra, src/r4dcaspt2_tra.F90:4-482:
 * fockcasci, fockdiag/tracic, calce0, intra_1/2/3 and solve_A..H_subspace).
 * e2_sub[8], sumc2_sub[8]: per-subspace E2 and c^2 in the order A..H (0 for skipped
 * subspaces); skip_mask bit k (k = 0 for A .. 7 for H) skips subspace k the way a
 * caspt2_restart file does (src/module_restart_file.F90:15-24).
 * *e0_out = sum_w eps_w D_ww (calce0.F90), *etotal_out = e2all + eigen(selectroot)
 * - eshift*sumc2 (r4dcaspt2_tra.F90:437-442). */
int dcg_caspt2(dcg_ctx *ctx, uint32_t skip_mask, double e2_sub[8], double sumc2_sub[8],
               double *e0_out, double *etotal_out);

/* Per-irrep energies of the last dcg_caspt2: the e2X(isym) lines that solve_A..G_subspace
 * print before their totals (solve_A_subspace.F90:262, solve_B_subspace.F90:268,
 * solve_C_subspace.F90:263, solve_D_subspace.F90:285, solve_E_subspace.F90:259,
 * solve_F_subspace.F90:284, solve_G_subspace.F90:273; the e2(isym) of e.g.
 * solve_A_subspace.F90:256).  All three arrays are e2_sym[8][nsym] in C order, index
 * k * nsym + isym - 1 for subspace k = 0 (A) .. 7 (H); Fortran reads them as (nsym, 8).
 * printed is 1 where the reference prints the line: a symmetry block with dimn > 0 whose S
 * keeps dimm > 0 vectors above the linear-dependence cutoff (solve_A_subspace.F90:118,158-164);
 * H prints no per-irrep lines, so its row stays 0.  sumc2_sym holds each block's share of
 * sumc2,X (not printed by the reference).  Any output may be NULL; nsym must equal the
 * system's nsymrpa.  DCG_E_STATE before the first dcg_caspt2. */
int dcg_caspt2_irreps(const dcg_ctx *ctx, int32_t nsym, double *e2_sym, double *sumc2_sym, int32_t *printed);

/* The CASCI determinants of the last dcg_casci as the bit strings the reference keeps in
 * dict_cas_idx (search_cas_configuration.F90:33-56, module_dict.F90:246-260): bit t-1 set when
 * active spinor t is occupied, in the reference's index order (ascending bit strings through
 * Gosper's hack, RAS and totsym filtered), which is also the row order of the CI coefficients
 * dcg_casci returns and of the dict records of CIDATA_sym<n> (casci.F90:118-160).  n >= ndet. */
int dcg_casci_determinants(const dcg_ctx *ctx, int64_t *dets_out, int32_t n);

/* H subspace on a caller-supplied, device-resident transformed H class (replaces
 * solve_H_subspace, src/solve_H_subspace.F90:23-191): with V = (ai|bj) - (aj|bi),
 * e = eps_a + eps_b - eps_i - eps_j + eshift, over a > b, i > j whose symmetry product
 * MULTB_S(MULTB_D(irp_a, irp_i), MULTB_D(irp_b, irp_j)) is 1:
 *   out[0] = e2h = -sum |V|^2 / e,  out[1] = sumc2,h = sum |V/e|^2.
 * Device inputs: hclass (ns, ni, ns, ni) complex column-major ((a i|b j) at
 * a + ns*(i + ni*(b + ns*j)), local indices), eps_i[ni], eps_s[ns], irp_i[ni], irp_s[ns]
 * (1-based irreps), multb_d and multb_s (nsymrpa x nsymrpa, [a-1][b-1] row-major,
 * 1-based values).  out is a host array.  Partial sums live in the context workspace. */
int dcg_solve_h(dcg_ctx *ctx, const void *hclass, int32_t ninact, int32_t nsec, const double *eps_i,
                const double *eps_s, const int32_t *irp_i, const int32_t *irp_s, const int32_t *multb_d,
                const int32_t *multb_s, int32_t nsymrpa, double eshift, double out[2]);

/* dcg_solve_h without any device allocation, for callers that cannot allocate device
 * memory themselves (a host program whose device memory all comes from its own pool or
 * from another runtime's allocator).  This entry point has no counterpart in the
 * reference.  Same inputs and result as dcg_solve_h, run on `stream` (a cudaStream_t,
 * NULL = default stream) of the current device, without a context.  Its partial sums live
 * in a file-scope device array of the library sized for ninact <= 128 (8128 inactive
 * pairs, 127 KiB), which every device that loads the library keeps until the process
 * exits; ninact > 128 returns DCG_E_ARG.  Every call looks up the array's device address in
 * the CUDA context current at the call, so it works in the device's primary context, in a
 * context of the caller's own and after cudaDeviceReset.  The call is synchronous (it reads
 * the result back into `out` and waits for `stream`): do not make it while `stream`, or in
 * global capture mode any stream, is being captured.  An error the caller left pending
 * returns DCG_E_CUDA without being cleared.  All calls share the array: calls that overlap
 * on the GPU race on it and must be serialised by the caller. */
int dcg_solve_h_noalloc(const void *hclass, int32_t ninact, int32_t nsec, const double *eps_i,
                        const double *eps_s, const int32_t *irp_i, const int32_t *irp_s,
                        const int32_t *multb_d, const int32_t *multb_s, int32_t nsymrpa, double eshift,
                        void *stream, double out[2]);

/* Orbital energies after fockdiag (eps, nmo entries, CAS order). */
int dcg_get_eps(const dcg_ctx *ctx, double *eps_out, int32_t n);

/* Per-stage device times of the last dcg_casci/dcg_caspt2 (ms), in the order:
 * 0 integral expansion, 1 CASCI matrix, 2 CASCI eigensolve, 3 Fock build+diag,
 * 4 CI rotation, 5 RDMs, 6 transformation, 7..14 subspaces A..H (their builds and own
 * solves), 15 the joint eigensolves of the A and C blocks that go through the Gram factor,
 * 16 the joint S and B' eigensolves and E2 of the B, D, E, F and G blocks.  Returns the
 * count. */
int dcg_stage_times(const dcg_ctx *ctx, double *ms_out, int32_t n);

/* Device kernel launches issued by the last dcg_set_system+dcg_casci+dcg_caspt2. */
int64_t dcg_kernel_launches(const dcg_ctx *ctx);

/* Library self-description (build string). */
const char *dcg_version(void);

/* The context's CUDA stream (a cudaStream_t), so a caller can order or time its own work
 * against the library's. */
void *dcg_stream(const dcg_ctx *ctx);

/* Hermitian eigendecomposition on the device, the solver behind every ZHEEV/DSYEV call of
 * the path (src/diag.F90:43,109): ascending eigenvalues w_out[n] and, when z_re is not
 * NULL, the eigenvectors as columns of z_re/z_im (n x n, column-major; z_im may be NULL to
 * drop the imaginary plane).  The upper triangle of a_re/a_im (column-major; a_im NULL for a
 * real symmetric matrix) is read, as ZHEEV with uplo='U' reads it. */
int dcg_heev(dcg_ctx *ctx, int32_t n, const double *a_re, const double *a_im, double *w_out, double *z_re,
             double *z_im);
/* Several Hermitian eigendecompositions in one batch (nmat <= 32): their tridiagonal reductions
 * run together in one launch, as the subspace solvers batch their S and B' matrices.  Per
 * matrix q: dimension n[q], upper triangle of a_re[q]/a_im[q] (a_im or a_im[q] NULL: real),
 * eigenvalues w_out[q] (ascending) and, when z_re and z_re[q] are not NULL, all eigenvectors. */
int dcg_heev_batch(dcg_ctx *ctx, int32_t nmat, const int32_t *n, const double *const *a_re,
                   const double *const *a_im, double *const *w_out, double *const *z_re, double *const *z_im);

/* dcg_heev returning only the eigenvectors of eigenvalues vlo..n-1 (ascending), as the
 * columns of z_re/z_im (n x (n - vlo)): the S-matrix use, which keeps the eigenvectors above
 * the linear-dependence cutoff, and the CASCI use, which keeps the lowest roots. */
int dcg_heev_range(dcg_ctx *ctx, int32_t n, const double *a_re, const double *a_im, double *w_out, int32_t vlo,
                   double *z_re, double *z_im);

/* Symmetric tridiagonal eigendecomposition (the divide-and-conquer stage of dcg_heev; the
 * role of LAPACK's DSTEDC): diagonal d[n], off-diagonal e[n-1] (host arrays), ascending
 * eigenvalues w_out[n] and, when z_out is not NULL, eigenvectors as the columns of z_out
 * (n x n, column-major). */
int dcg_stedc(dcg_ctx *ctx, int32_t n, const double *d, const double *e, double *w_out, double *z_out);

/* Complex GEMM on device buffers at a chosen precision (the contraction kernel of the
 * 4-index transformation): for z < batch, i < M, j < N
 *   C[z*c_sb + i*c_si + j*c_sj] (+)= sum_{k<K} A[z*a_sb + i*a_si + k*a_sk] * op(B)(k, j)
 * with op(B)(k, j) = B[k + j*ldb], conjugated when conj_b; strides count complex elements
 * (double2).  DCG_PREC_SPLIT runs the BF16 tensor-core path with FP64 recombination (any
 * strides; five slices per operand, ~2^-36 of max|row of A| max|column of op(B)| per term),
 * DCG_PREC_SPLIT_ACC the same with seven slices (~2^-45); DCG_PREC_FP64 needs a_si = c_si = 1.
 * accumulate != 0 adds to C. */
int dcg_zgemm(dcg_ctx *ctx, int precision, int32_t M, int32_t N, int32_t K, int32_t batch, const void *A, int64_t a_si,
              int64_t a_sk, int64_t a_sb, const void *B, int64_t ldb, int32_t conj_b, void *C, int64_t c_si,
              int64_t c_sj, int64_t c_sb, int32_t accumulate);

/* Kernel families whose launches can be timed with CUDA events on the context stream. */
#define DCG_FAM_NONE 0
#define DCG_FAM_TRANSFORM 1   /* 4-index transformation GEMMs; work = FLOPs (complex MAC = 8)  */
#define DCG_FAM_HSTREAM 2     /* H-subspace streaming reduction; work = bytes it must read: the a > b
                                 half of the H class, C(ns,2) ni (ni-1) complex values          */
#define DCG_FAM_RDM 3         /* density GEMMs; work = FLOPs                                     */
#define DCG_FAM_SCATTER 4     /* record expansion; work = record bytes read                      */
#define DCG_FAM_EIG 5         /* Hermitian eigensolver launches; work = nominal FLOPs 16/3 n^3   */
#define DCG_FAM_EIG_TRI 6     /* eigensolver phases: tridiagonal reduction (FLOPs 16/3 n^3)      */
#define DCG_FAM_EIG_VAL 7     /*   tridiagonal divide and conquer (values and vectors; 4/3 n^3)  */
#define DCG_FAM_EIG_VEC 8     /*   reserved (no launches)                                          */
#define DCG_FAM_EIG_BACK 9    /*   back-transformation (FLOPs 8 n^2 m)                            */
#define DCG_FAM_SPLIT_MMA 10  /* tcgen05 split-precision GEMM kernel; work = BF16 tensor FLOPs      */

/* Time limit of the context's device-side waits that can give up: the grid barriers and the
 * published-reflector waits of the Householder tridiagonalisation (default 5 s) and the
 * pipeline waits of the tensor-core GEMM kernels (default 2 s).  A wait that runs out sets an
 * error flag; the kernel's other blocks leave at their next wait, copies still in flight land
 * and issued tensor-core operations complete (waits bounded by the default limits) before a
 * block frees its tensor memory and returns, and the call returns DCG_E_NUMERIC with the
 * reason in dcg_last_error.  The context stays usable.  seconds = 0 restores the defaults;
 * values in (0, 60] set the limit.  A diagnostic and fault-test hook: a short limit makes
 * ordinary waits run out. */
int dcg_set_wait_limit(dcg_ctx *ctx, double seconds);

/* Select the family timed during subsequent calls (DCG_FAM_NONE disables; resets stats). */
int dcg_time_family(dcg_ctx *ctx, int32_t family);
/* Accumulated device time (ms), launch count and algorithmic work of the timed family. */
int dcg_family_stats(const dcg_ctx *ctx, double *ms, int64_t *launches, double *work);

/* CASCI eigensolver of dcg_casci.  AUTO: dense Householder + divide-and-conquer (the ZHEEV
 * of diag.F90:66-128) below 600 determinants or for more than 12 roots, block Davidson on the
 * resident Hamiltonian otherwise (residual norms <= 1e-13 max(1, max |H_ii|) for every
 * returned root).  DENSE / DAVIDSON force one of them (DAVIDSON needs ndet >= roots + 5). */
#define DCG_CASCI_AUTO 0
#define DCG_CASCI_DENSE 1
#define DCG_CASCI_DAVIDSON 2
int dcg_set_casci_solver(dcg_ctx *ctx, int32_t solver);
/* Davidson iterations of the last dcg_casci (0 when the dense solver ran). */
int32_t dcg_casci_iterations(const dcg_ctx *ctx);

/* Solver of the A and C blocks that go through the (nelec +- 1)-electron Gram factor G
 * (S = G^H G, metric K = G G^H).  AUTO: when no eigenvalue of K falls under the 1e-8 cutoff
 * of cutoff.F90:37-70 (so X spans the range of G^H), E2 and c^2 come from one Cholesky solve
 * u = K^-1 G v as -u^H (D + alpha)^-1 u and |(D + alpha)^-1 u|^2, equal to the reference's
 * sums over the eigenpairs of B'; when r <= 64 eigenvalues fall under it, from the same solve
 * on the complement of their r eigenvectors (deflated metric, compression of D + alpha);
 * otherwise, and always with EIGEN, from the eigendecompositions of K and B'. */
#define DCG_METRIC_AUTO 0
#define DCG_METRIC_EIGEN 1
int dcg_set_metric_solver(dcg_ctx *ctx, int32_t solver);
/* Gram blocks the last dcg_caspt2 solved by the Cholesky route (deflated or not), and those
 * of them with eigenvalues under the cutoff deflated. */
int32_t dcg_gram_cholesky_blocks(const dcg_ctx *ctx);
int32_t dcg_gram_deflated_blocks(const dcg_ctx *ctx);

/* Device bytes the context holds: its grow-only workspace (integral classes, CI vectors,
 * densities, subspace matrices, solver scratch), which stays resident between solves. */
int64_t dcg_device_bytes(const dcg_ctx *ctx);
/* Release the context's device workspace and system; the next solve starts with
 * dcg_set_system again. */
int dcg_trim(dcg_ctx *ctx);
/* Upper estimate of the device bytes one set_system + casci + caspt2 of sys needs in a fresh
 * context of either precision (the admission size of the serving loop; host pointers of sys
 * are not read). */
int64_t dcg_footprint_estimate(const dcg_system *sys);

/* ------------------------------------------------------------------------ serving loop
 * A server runs independent CASCI/CASPT2 solves (each one .caspt2_ciroots entry of one
 * system: dcg_set_system + dcg_casci(selectroot roots) + dcg_caspt2) from a request queue on
 * one GPU.  It owns `slots` contexts, one host worker thread and one CUDA stream each, so the
 * solves of different requests overlap on the device.  A free slot takes the first queued
 * request whose dcg_footprint_estimate fits the HBM budget beside the bytes the other slots
 * hold (the running requests' estimates and the idle slots' resident workspaces; an idle slot
 * releases its workspace when a queued request does not fit).  The host arrays a request's
 * dcg_system points at must stay valid until its result has been polled. */
typedef struct dcg_server dcg_server;

typedef struct dcg_request_result {
    uint64_t request_id;
    int32_t status;          /* DCG_OK or the failing call's status                       */
    int32_t ndet;            /* CASCI determinants                                        */
    double casci_energy;     /* energy of the selected root (casci.F90 root selectroot)   */
    double e2[8], sumc2[8];  /* subspaces A..H                                            */
    double e0, etotal;       /* as dcg_caspt2                                              */
    double t_submit, t_start, t_end;   /* seconds on the server clock (dcg_server_clock)  */
    int32_t slot;            /* worker slot that ran the request                          */
    int32_t attempts;        /* 1, or 2 when a first attempt ran out of device memory     */
    char error[96];          /* the failing call's dcg_last_error (empty on success)      */
} dcg_request_result;

/* slots in 1..64; hbm_budget_bytes <= 0 takes 90% of the device's free memory at creation. */
int dcg_server_create(int device, int precision, int32_t slots, int64_t hbm_budget_bytes, dcg_server **out);
/* Queue one request (DCG_E_NOMEM when its estimate exceeds the whole budget). */
int dcg_server_submit(dcg_server *srv, const dcg_system *sys, uint64_t request_id);
/* Take one finished request, waiting up to timeout_ms; returns 1 when none finished in time. */
int dcg_server_poll(dcg_server *srv, int32_t timeout_ms, dcg_request_result *out);
/* Requests waiting in the queue and running on the slots. */
int dcg_server_pending(dcg_server *srv, int32_t *queued, int32_t *running);
/* The server clock (seconds, monotonic) of the result stamps. */
double dcg_server_clock(const dcg_server *srv);
/* Device bytes held by the server's slots now (their contexts' workspaces). */
int64_t dcg_server_device_bytes(dcg_server *srv);
/* Drop queued requests, finish the running ones, join the workers and free the contexts. */
int dcg_server_destroy(dcg_server *srv);

/* Merged eigensolver reductions.  A context with on != 0 hands its batched Householder
 * reductions (the cooperative kernel that reduces the S, metric and B' matrices of a solve, the
 * role of the ZHETRD inside the ZHEEV calls of diag.F90:66-128) to a per-device batcher: the
 * submissions of all such contexts that wait at the same time run as one cooperative launch,
 * each matrix with its own block group and barrier, so concurrent requests overlap their
 * barrier-bound column loops instead of queueing for the GPU one after the other.  A matrix's
 * result is the same bits alone and merged.  The serving slots set it; other contexts do not
 * by default. */
int dcg_set_merge_reductions(dcg_ctx *ctx, int32_t on);
/* Counters of the merged reductions on `device` since the process started: out[0] launches,
 * out[1] launches that carried more than one context's reductions, out[2] submissions carried. */
int dcg_merged_reduction_stats(int device, int64_t out[3]);

/* The CASCI check of e0test (e0test.F90:4-272, called by r4dcasci.F90:89) for the selected
 * root of the last dcg_casci: out[0..1] energyHF(1), energyHF(2) of the lowest
 * ninact + nelec spinors; out[2..5] energy 1..4 (inactive one- and two-electron, active
 * one-electron with the inactive mean field, active two-electron); out[6] their sum;
 * out[7] eigen - ecore - out[6] (the printed "error"). */
int dcg_casci_energy_check(dcg_ctx *ctx, double out[8]);

/* ------------------------------------------------------------------------ autotuner
 * Shape-dependent launch choices (today: the tile shape, 64x64, 32x128 or 128x32, and the
 * K-split of the FP64 GEMMs; for the split-precision tensor-core GEMMs the kernel, one tile
 * per CTA or persistent CTAs whose epilogue overlaps the next tile's MMAs, and the CTA
 * raster, row-block or column-block major, which decides which operand tiles meet in L2) are
 * tuned on first use, for products of at least ~1 ms of work:
 * every candidate is timed with CUDA events on the calling context's stream and the fastest
 * is kept in a process-wide table that every context then uses.  Different choices change
 * only the summation order of the products.
 * With the environment variable DCG_TUNE_FILE naming a text file, the table is read from it
 * at first use and each new entry appended to it, so later processes reuse the choices.
 * mode: 1 tune (default; environment DCG_AUTOTUNE=0 starts with 0), 0 use the built-in
 * heuristics for keys not yet tuned, 2 clear the table (mode unchanged), other values only
 * query.  Returns the mode before the call. */
typedef struct dcg_tune_entry {
    int32_t kind;                 /* 1: FP64 GEMM tile and K-split, 2: split GEMM kernel/raster */
    int32_t ops, m, n, k, flags;  /* the decision's key (ops: op codes or batch; flags:
                                     upper + 2 batch for the FP64 GEMM)                    */
    int32_t choice, ncand;        /* chosen candidate (0 = the heuristic) of ncand           */
    float best_ms, heuristic_ms;  /* measured time of the choice and of the heuristic        */
} dcg_tune_entry;

int dcg_autotune_mode(int32_t mode);
/* Per context: on = 0 makes the context use tuned entries and heuristics only, never running
 * trials itself (the serving loop's slots are created so). */
int dcg_set_autotune_trials(dcg_ctx *ctx, int32_t on);
/* Entries of the table (at most max_entries written to out); returns their total number. */
int32_t dcg_autotune_entries(dcg_tune_entry *out, int32_t max_entries);

/* ------------------------------------------------------------------------ IVO
 * Improved virtual orbitals (r4divo.F90:80-93, fockivo.F90:44-215) on the system of the last
 * dcg_set_system / dcg_set_system_mdcint (its ninact, nact, nsec, nelec as the IVO input
 * gives them): the Fock matrix of the secondary spinors
 *   f(a,b) = e_a delta_ab - sum_k w_k [(ab|kk) - (ak|kb)] / numh
 * over the numh highest active spinors k (w_k = 1/2 for the two highest when nelec is odd;
 * numh = nhomo, or for nhomo = 0 the spinors up to the last active one within 0.1 Eh of the
 * HOMO energy), diagonalised per abelian irrep block by the LAPACK ZHEEV algorithm (its
 * eigenvector signs included).  The blocks are, per fermion-irrep group (nfsym = 2 with
 * inversion symmetry), every second irrep: 1, 3, .. nsymrpa/2 and nsymrpa/2+1, .. nsymrpa.
 *   mo_energy : nmo orbital energies, CAS order (dcg_mrconee.mo_energy)
 *   eps       : nsec, the eigenvalue at each block position (0 outside the blocks)
 *   u_re/u_im : nsec x nsec column-major, U(a_i, a_j) = V(i, j) of the block of a_i and a_j
 *   block_isym: nsec, the irrep of the block each secondary spinor belongs to, 0 if none
 * Any output may be NULL. */
int dcg_ivo(dcg_ctx *ctx, int32_t nfsym, const double *mo_energy, int32_t nhomo, double *eps, double *u_re,
            double *u_im, int32_t *block_isym, int32_t *numh_out);

/* ------------------------------------------------------------------------ DIRAC files
 * Host readers of DIRAC's MRCONEE and MDCINT files, so a process without the Fortran driver
 * can fill dcg_system / dcg_mdcint_raw.  They need no GPU and no context; on failure they
 * return DCG_E_IO or DCG_E_ARG with the reason in dcg_io_last_error() (per thread). */
typedef struct dcg_active_input {
    int32_t ninact, nact, nsec, nelec;   /* .ninact .nact .nsec .nelec                          */
    int32_t diracver;                    /* .diracver: >= 21 flips the sign of Im h
                                            (read_mrconee.F90:579-581)                           */
    int32_t scheme;                      /* .scheme; 0 = the default of .diracver: 4 above 22,
                                            else 6 (read_input_module.F90:986-1011)              */
    int32_t nras1, nras2, nras3;         /* .ras1/.ras2/.ras3 list lengths (all 0: CAS)         */
    const int32_t *ras1, *ras2, *ras3;   /* ascending energy-order spinor numbers, 1-based      */
} dcg_active_input;

/* MRCONEE (read_mrconee.F90:226-600): energy-order sort, optional RAS order
 * (read_mrconee.F90:602-715), Kramers pairing by exactly equal orbital energies
 * (read_mrconee.F90:515-530), one-electron integrals in CAS order. */
typedef struct dcg_mrconee {
    int32_t nmo, nsymrpa;
    int32_t dirac_32bit;                 /* 1: 32-bit integers detected (read_mrconee.F90:1-222) */
    double ecore, hf_energy;
    int32_t *multb;                      /* MULTB(2n,2n) column-major, 1-based values            */
    int32_t *irpamo;                     /* nmo, CAS order                                       */
    double *mo_energy;                   /* nmo, CAS order (caspt2_mo_energy)                    */
    int32_t *dirac_to_cas, *cas_to_dirac;   /* nmo + 1, 1-based, entry 0 unused                 */
    double *h_re, *h_im;                 /* (nmo, nmo) column-major, CAS order                   */
} dcg_mrconee;

int dcg_read_mrconee(const char *path, const dcg_active_input *inp, dcg_mrconee **out);
void dcg_free_mrconee(dcg_mrconee *m);

/* MDCINT, MDCINXXXX1, MDCINXXXX2, ... of `directory` (get_filename.F90:1-41) as the flattened
 * record stream of dcg_mdcint_raw (create_newmdcint.F90:3-171's reads; real-only detected from
 * the record length as module_realonly.F90:29-77 does).  pinned = 1 places the entry arrays in
 * page-locked memory (cudaHostAlloc), so dcg_set_system_mdcint copies them at link speed. */
int dcg_read_mdcint(const char *directory, const dcg_mrconee *mrc, const dcg_active_input *inp, int32_t pinned,
                    dcg_mdcint_raw **out);
void dcg_free_mdcint(dcg_mdcint_raw *raw);

const char *dcg_io_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* DCASPT2_GB300_H */
