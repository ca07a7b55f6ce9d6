// Launch wrappers shared between the translation units of the library.
#pragma once
#include "dcg_common.cuh"

namespace dcg {

// ---- dcg_ci.cu
void upload_binomials(Context &c);
void launch_casmat(Context &c, const uint64_t *dets, int ndet, const cplx *h, const cplx *g, cplx *H);
void launch_apply_E(Context &c, int na, int64_t M, const uint64_t *full, const cplx *x, int nv, cplx *out);
void launch_occ_energy(Context &c, int na, int64_t M, const uint64_t *full, const double *eps_act, const cplx *psi,
                       cplx *psit);
void launch_embed(Context &c, int ndet, const int64_t *pos, const cplx *cvec, cplx *psi, int64_t M);
void launch_detsc(Context &c, const uint64_t *dets, int ndet, const cplx *Uact, cplx *ds);

// Gram factor G (Mp x dimn) of the A (create = 1) or C (create = 0) overlap matrix
void launch_gram(Context &c, int na, int64_t Mp, const uint64_t *dets_p, int64_t M, const cplx *Y, const int *ind,
                 int dimn, int create, cplx *G);
// A(i, j) *= s[soff + i] (or /= when inv)
void launch_scale_rows(Context &c, int m, int n, cplx *A, int64_t lda, const double *s, int soff, bool inv);

// ---- dcg_ints.cu
// Dense class tensors of the two-electron integrals in the original spinor basis.
enum ClassId {
    CL_C1 = 0, CL_C2, CL_C3, CL_D1, CL_D2, CL_D3, CL_E, CL_F, CL_G, CL_H,
    CL_F1A, CL_F2A, CL_F1D, CL_F2D, CL_COUNT
};
struct ClassTensor {
    cplx *p = nullptr;
    int sp[4] = {0, 0, 0, 0};   // spaces 1 inact, 2 act, 3 sec
    int dim[4] = {0, 0, 0, 0};
    int64_t size = 0;
    int diag = 0;               // 0 full; 1: (a,b,k,k) stored [a,b,k]; 2: (a,k,k,b) stored [a,b,k]
};
void class_layout(const Context &c, ClassTensor cls[CL_COUNT]);
void launch_scatter(Context &c, const int32_t *ijkl, const cplx *val, int64_t nrec, cplx *inttw,
                    ClassTensor cls[CL_COUNT]);
void launch_fock(Context &c, const cplx *h, const cplx *g, const ClassTensor cls[CL_COUNT], const cplx *D1act,
                 cplx *f);
// core Fock pieces in the original basis: Fai(act,inact), Fsi(sec,inact), Fsa(sec,act) (Fsa already minus
// sum_q (aq|qp) over active q)
void launch_core_fock(Context &c, const cplx *h, const cplx *g, const ClassTensor cls[CL_COUNT], cplx *Fai, cplx *Fsi,
                      cplx *Fsa);
// 4-index sub-block of inttw: out(i,j,k,l) = g(o1+i, o2+j, o3+k, o4+l)
void launch_subblock(Context &c, const cplx *g, int nmoc, const int off[4], const int dim[4], cplx *out);
// zero entries with |x| < thr
void launch_zero_small(Context &c, cplx *x, int64_t n, double thr);
// out(i,j) = A(idx[i], idx[j]) with lda
void launch_gather2(Context &c, const cplx *A, int64_t lda, const int *idx, int n, cplx *out);
// A(idx[i], idx[j]) = X(i,j)
void launch_scatter2(Context &c, const cplx *X, int n, const int *idx, cplx *A, int64_t lda);
void launch_scale_cols(Context &c, cplx *Z, int64_t ldz, int n, int m, const double *w, int woff);

// ---- dcg_pt2.cu
struct RDMView {
    const cplx *g1, *g2, *g3;   // <E>, <EE>, <EEE>
    const cplx *t1, *t2, *t3;   // same with F = sum_w eps_w E_ww rightmost
    int na;
};
void launch_SB(Context &c, char sub, const RDMView &r, const int *ind, int dimn, const double *eps_act, double e0,
               cplx *S, cplx *B);
void launch_gather_v(Context &c, const cplx *V, const int64_t *outer_off, int nouter, const int64_t *inner_off,
                     int dimn, cplx *Vsel);
void launch_e2(Context &c, const cplx *VC, int dimm, int nouter, const double *alpha, const double *wb, double *e2o,
               double *sc2o);
void launch_v_B(Context &c, const RDMView &r, const cplx *Bc, int ni, cplx *V);
void launch_v_D(Context &c, const RDMView &r, const cplx *D1c, const cplx *D2c, const cplx *effh, int ni, int ns,
                cplx *V);
void launch_v_E(Context &c, const RDMView &r, const cplx *Ec, int ni, int ns, cplx *V);
void launch_v_G(Context &c, const RDMView &r, const cplx *Gc, int ni, int ns, cplx *V);
// permutations feeding the A / C / F V-build GEMMs
void launch_perm_A(Context &c, const RDMView &r, cplx *P3, cplx *unused);
void launch_perm_C2(Context &c, const RDMView &r, cplx *P3, cplx *P2);
void launch_perm_F(Context &c, const RDMView &r, cplx *P2, cplx *unused);
void launch_permute_A1(Context &c, const cplx *A1, int na, int ni, cplx *A1p);
void launch_v_A_rest(Context &c, const RDMView &r, const cplx *A1, const cplx *effh, int ni, cplx *V);
void launch_F_pack(Context &c, const cplx *Fc, int ns, int na, cplx *Fp);
// partial sums launch_h_stream2 writes (h_stream_blocks(ni, ns) of each)
int h_stream_blocks(int ni, int ns);
void launch_h_stream2(Context &c, const cplx *Hc, int ni, int ns, const double *eps_i, const double *eps_s,
                      const int *irp_i, const int *irp_s, const int *md, const int *msy, int nsym, double eshift,
                      double *e2part, double *sc2part);

}  // namespace dcg
