// DIRAC's MDCINT records to the MDCINTNEW stream on the device: the canonicalisation of
// create_newmdcint (create_newmdcint.F90:3-321), which the reference runs on the host through
// scratch files.  Every MDCINT entry (k l | of a record (ikr jkr |) stands for up to four
// candidates: the record and its time-reversed partner (n = 1, 2; create_newmdcint.F90:
// 206-217), each also with its bra and ket exchanged when the file stores only one of a
// (ij|kl) / (ji|lk) pair (schemes other than 6 with |ikr| != |jkr|; 219-246).  A candidate is
// mapped to CAS order through the header's Kramers table and the DIRAC-to-CAS map and kept when
// its Kramers partners pass the TYPE1-4 filter (286-320) and its value exceeds the 0.25e-12
// cutoff; kept candidates are written as (i~, j~, k~, l~) with the value Re - i Im
// (171-177), in the order the reference writes them (record, n, exchange, entry).
//
// Two passes per record (one block each): count the kept candidates, then, after an
// exclusive scan of the record counts, write them in order (a block-wide prefix sum per chunk
// of 1024 candidates).  Integer work and byte moves, bound by the entry stream.
#include <algorithm>
#include <numeric>
#include <vector>

#include "dcg_common.cuh"

namespace dcg {

namespace {

constexpr int MC_THREADS = 1024;

struct McArgs {
    const int64_t *rec_off;   // nrec + 1
    const int32_t *ikr, *jkr;  // per record
    const int32_t *indk, *indl;
    const double *re, *im;     // im may be null (real-only)
    const int32_t *kr;         // kr[o + x] for x in [-nkr, nkr], o = nkr
    int nkr;
    const int32_t *d2c;        // nmo + 1, 1-based DIRAC -> CAS
    int nmo;
    int scheme, realonly;
};

__device__ __forceinline__ int kr_signed(int x) { return ((x & 1) ? 1 : -1) * (x / 2 + x % 2); }
__device__ __forceinline__ int swapkr(int x) { return (x & 1) ? x + 1 : x - 1; }

// Candidate q of record r (q < 2 reps nz: n = q / (reps nz), rep = (q / nz) % reps, entry
// q % nz): kept?  When kept, its CAS indices and value.
__device__ bool candidate(const McArgs &a, int64_t r, int64_t q, int reps, int64_t nz, int32_t out[4], double &vre,
                          double &vim) {
    const int n = (int)(q / (reps * nz));
    const int rep = (int)((q / nz) % reps);
    const int64_t e = a.rec_off[r] + q % nz;
    int ci = a.ikr[r], cj = a.jkr[r], ck = a.indk[e], cl = a.indl[e];
    double rr = a.re[e], ri = a.im ? a.im[e] : 0.0;
    if (n == 1) {   // time-reversed partner (create_newmdcint.F90:206-217)
        const long long prod = (long long)ci * cj * (long long)ck * cl;
        const double sgn = prod >= 0 ? 1.0 : -1.0;
        ci = -ci;
        cj = -cj;
        ck = -ck;
        cl = -cl;
        rr = -rr * sgn;
        ri = ri * sgn;
    }
    const bool big = a.realonly ? fabs(rr) > 0.25e-12 : (fabs(rr) > 0.25e-12 || fabs(ri) > 0.25e-12);
    if (!big) return false;
    double vr = rr, vi = ri;
    if (rep == 1) {   // bra and ket exchanged (219-246)
        int t = ci;
        ci = cj;
        cj = t;
        t = ck;
        ck = cl;
        cl = t;
        const bool t23 = (((ci < 0) + (cj < 0)) == 1) && (((ck < 0) + (cl < 0)) == 1);
        if (t23) {
            ci = -ci;
            cj = -cj;
            ck = -ck;
            cl = -cl;
        }
        if (!a.realonly && !t23) vi = -vi;
    }
    const int o = a.nkr;
    if (ci < -o || ci > o || cj < -o || cj > o || ck < -o || ck > o || cl < -o || cl > o) return false;
    const int di = a.kr[o + ci], dj = a.kr[o + cj], dk = a.kr[o + ck], dl = a.kr[o + cl];
    if (di < 1 || di > a.nmo || dj < 1 || dj > a.nmo || dk < 1 || dk > a.nmo || dl < 1 || dl > a.nmo) return false;
    const int i = a.d2c[di], j = a.d2c[dj], k = a.d2c[dk], l = a.d2c[dl];
    const int ik = kr_signed(i), jk = kr_signed(j), kk_ = kr_signed(k), lk = kr_signed(l);
    const int ii = abs(ik), jj = abs(jk), kk = abs(kk_), ll = abs(lk);
    const bool t1 = ik > 0 && jk > 0 && kk_ > 0 && lk > 0;
    const bool t2 = ik > 0 && jk < 0 && kk_ > 0 && lk < 0;
    const bool t3 = ik > 0 && jk < 0 && kk_ < 0 && lk > 0;
    const bool t4 = ik > 0 && jk < 0 && kk_ < 0 && lk < 0;
    const bool c1 = (ii <= jj && kk <= ll && (ii < kk || (ii == kk && jj <= ll))) ||
                    (ii <= jj && ll <= kk && (ii < ll || (ii == ll && jj <= kk)));
    const bool c23 = ii <= jj && kk <= ll && (ii < kk || (ii == kk && jj <= ll));
    const bool keep = (t1 && c1) || (t2 && c23) || (t3 && c23) || (t4 && ii <= jj);
    if (!keep) return false;
    out[0] = swapkr(i);
    out[1] = swapkr(j);
    out[2] = swapkr(k);
    out[3] = swapkr(l);
    vre = vr;
    vim = a.realonly ? 0.0 : -vi;   // Re - i Im
    return true;
}

__device__ __forceinline__ int reps_of(const McArgs &a, int64_t r) {
    return (a.scheme != 6 && abs(a.ikr[r]) != abs(a.jkr[r])) ? 2 : 1;
}

// counts[r] = kept candidates of record r (one block per record).
__global__ void __launch_bounds__(MC_THREADS) mdcint_count_kernel(McArgs a, int64_t *counts) {
    __shared__ int64_t red[MC_THREADS / 32];
    const int64_t r = blockIdx.x;
    const int64_t nz = a.rec_off[r + 1] - a.rec_off[r];
    const int reps = reps_of(a, r);
    int64_t cnt = 0;
    for (int64_t q = threadIdx.x; q < 2 * reps * nz; q += blockDim.x) {
        int32_t o4[4];
        double vr, vi;
        cnt += candidate(a, r, q, reps, nz, o4, vr, vi) ? 1 : 0;
    }
    for (int s = 16; s > 0; s >>= 1) cnt += __shfl_down_sync(0xffffffffu, cnt, s);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
        counts[r] = t;
    }
}

// Kept candidates of record r written from base[r] on, in candidate order (block prefix sums
// over chunks of blockDim candidates).
__global__ void __launch_bounds__(MC_THREADS) mdcint_write_kernel(McArgs a, const int64_t *base, int32_t *ijkl,
                                                                  double *vre, double *vim) {
    __shared__ int wsum[MC_THREADS / 32];
    __shared__ int64_t run;
    const int64_t r = blockIdx.x;
    const int64_t nz = a.rec_off[r + 1] - a.rec_off[r];
    const int reps = reps_of(a, r);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (threadIdx.x == 0) run = base[r];
    __syncthreads();
    for (int64_t q0 = 0; q0 < 2 * reps * nz; q0 += blockDim.x) {
        const int64_t q = q0 + threadIdx.x;
        int32_t o4[4];
        double vr = 0.0, vi = 0.0;
        const bool kept = q < 2 * reps * nz && candidate(a, r, q, reps, nz, o4, vr, vi);
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
            const int64_t p = run + before;
            ijkl[4 * p + 0] = o4[0];
            ijkl[4 * p + 1] = o4[1];
            ijkl[4 * p + 2] = o4[2];
            ijkl[4 * p + 3] = o4[3];
            vre[p] = vr;
            vim[p] = vi;
        }
        __syncthreads();
        if (threadIdx.x == 0) run += total;
        __syncthreads();
    }
}

template <typename T>
T *up(Context &c, const std::string &name, const T *h, size_t n) {
    T *d = wsget<T>(c, name, n + 1);
    if (n) DCG_CUDA(cudaMemcpyAsync(d, h, sizeof(T) * n, cudaMemcpyHostToDevice, c.stream));
    return d;
}

}  // namespace

int64_t mdcint_canonicalize(Context &c, const dcg_mdcint_raw &raw, int32_t **ijkl_out, double **re_out,
                            double **im_out) {
    if (raw.nrec < 0 || raw.nent < 0 || raw.nkr < 0 || raw.nmo < 1 || !raw.rec_off || !raw.kr || !raw.dirac_to_cas)
        throw Error{DCG_E_ARG, "mdcint: inconsistent raw record description"};
    if (raw.nrec > 0 && (!raw.ikr || !raw.jkr || !raw.indk || !raw.indl || !raw.re))
        throw Error{DCG_E_ARG, "mdcint: missing entry arrays"};
    if (raw.rec_off[0] != 0 || raw.rec_off[raw.nrec] != raw.nent)
        throw Error{DCG_E_ARG, "mdcint: record offsets do not span the entries"};
    if (raw.nrec > 0x7fffffff) throw Error{DCG_E_ARG, "mdcint: too many records for one launch"};
    McArgs a;
    a.rec_off = up(c, "mdc.off", raw.rec_off, (size_t)raw.nrec + 1);
    a.ikr = up(c, "mdc.ikr", raw.ikr, (size_t)raw.nrec);
    a.jkr = up(c, "mdc.jkr", raw.jkr, (size_t)raw.nrec);
    a.indk = up(c, "mdc.k", raw.indk, (size_t)raw.nent);
    a.indl = up(c, "mdc.l", raw.indl, (size_t)raw.nent);
    a.re = up(c, "mdc.re", raw.re, (size_t)raw.nent);
    a.im = (raw.realonly || !raw.im) ? nullptr : up(c, "mdc.im", raw.im, (size_t)raw.nent);
    // kr[o + x], x = -nkr..nkr: kr(i) = raw.kr[2 (i-1)], kr(-i) = raw.kr[2 (i-1) + 1]; kr(0) = 0
    std::vector<int32_t> krt(2 * (size_t)raw.nkr + 1, 0);
    for (int i = 1; i <= raw.nkr; i++) {
        krt[raw.nkr + i] = raw.kr[2 * (i - 1)];
        krt[raw.nkr - i] = raw.kr[2 * (i - 1) + 1];
    }
    a.kr = up(c, "mdc.kr", krt.data(), krt.size());
    a.nkr = raw.nkr;
    a.d2c = up(c, "mdc.d2c", raw.dirac_to_cas, (size_t)raw.nmo + 1);
    a.nmo = raw.nmo;
    a.scheme = raw.scheme;
    a.realonly = raw.realonly ? 1 : 0;
    if (!raw.realonly && !raw.im) a.realonly = 1;
    int64_t *counts = wsget<int64_t>(c, "mdc.counts", (size_t)raw.nrec + 1);
    std::vector<int64_t> hc((size_t)raw.nrec), hb((size_t)raw.nrec + 1, 0);
    if (raw.nrec > 0) {
        mdcint_count_kernel<<<(unsigned)raw.nrec, MC_THREADS, 0, c.stream>>>(a, counts);
        DCG_LAUNCHED(c);
        DCG_CUDA(cudaMemcpyAsync(hc.data(), counts, sizeof(int64_t) * raw.nrec, cudaMemcpyDeviceToHost, c.stream));
        DCG_CUDA(cudaStreamSynchronize(c.stream));
    }
    for (int64_t r = 0; r < raw.nrec; r++) hb[r + 1] = hb[r] + hc[r];
    const int64_t nout = hb[raw.nrec];
    int32_t *ijkl = wsget<int32_t>(c, "mdc.ijkl", 4 * (size_t)nout + 4);
    double *vre = wsget<double>(c, "mdc.vre", (size_t)nout + 1);
    double *vim = wsget<double>(c, "mdc.vim", (size_t)nout + 1);
    if (nout > 0) {
        int64_t *base = up(c, "mdc.base", hb.data(), (size_t)raw.nrec);
        mdcint_write_kernel<<<(unsigned)raw.nrec, MC_THREADS, 0, c.stream>>>(a, base, ijkl, vre, vim);
        DCG_LAUNCHED(c);
    }
    DCG_CUDA(cudaStreamSynchronize(c.stream));
    *ijkl_out = ijkl;
    *re_out = vre;
    *im_out = vim;
    return nout;
}

}  // namespace dcg
