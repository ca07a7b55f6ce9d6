// Host readers of DIRAC's integral files: MRCONEE (one-electron part, orbital energies and
// irreps) and MDCINT / MDCINXXXX* (two-electron records), so that a serving process fills
// dcg_system and dcg_mdcint_raw without the Fortran driver.  Plain C++17 file parsing; the
// only CUDA call is the optional page-locked allocation of the MDCINT entry arrays.
//
// Fortran sequential unformatted files (gfortran layout): each record is a 4-byte length,
// the payload and the length again; a record above 2 GiB is split into sub-records whose
// leading marker is negative until the last one.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <set>
#include <string>
#include <vector>

#include "../../include/dcaspt2_gb300.h"

namespace {

thread_local std::string g_io_error;

struct IoError {
    int code;
    std::string msg;
};

std::vector<unsigned char> slurp(const std::string &path) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) throw IoError{DCG_E_IO, path + ": cannot open"};
    std::vector<unsigned char> d;
    if (std::fseek(f, 0, SEEK_END) == 0) {
        const long n = std::ftell(f);
        if (n > 0) {
            d.resize((size_t)n);
            std::fseek(f, 0, SEEK_SET);
            if (std::fread(d.data(), 1, d.size(), f) != d.size()) {
                std::fclose(f);
                throw IoError{DCG_E_IO, path + ": short read"};
            }
        }
    }
    std::fclose(f);
    return d;
}

// (offset, length) of each record's payload; continued records are joined into `joined`.
struct Records {
    std::vector<unsigned char> data;
    std::vector<std::vector<unsigned char>> joined;   // records that were split into sub-records
    std::vector<const unsigned char *> ptr;
    std::vector<size_t> len;
};

int32_t rd_i32(const unsigned char *p) {
    int32_t v;
    std::memcpy(&v, p, 4);
    return v;
}
int64_t rd_i64(const unsigned char *p) {
    int64_t v;
    std::memcpy(&v, p, 8);
    return v;
}
double rd_f64(const unsigned char *p) {
    double v;
    std::memcpy(&v, p, 8);
    return v;
}

Records read_records(const std::string &path) {
    Records r;
    r.data = slurp(path);
    const size_t n = r.data.size();
    size_t off = 0;
    std::vector<std::pair<size_t, size_t>> spans;
    std::vector<int> joined_idx;
    while (off < n) {
        std::vector<std::pair<size_t, size_t>> parts;
        for (;;) {
            if (off + 4 > n) throw IoError{DCG_E_IO, path + ": truncated record marker at byte " + std::to_string(off)};
            const int32_t lead = rd_i32(&r.data[off]);
            const size_t size = (size_t)(lead < 0 ? -(int64_t)lead : lead);
            if (off + 8 + size > n) throw IoError{DCG_E_IO, path + ": truncated record at byte " + std::to_string(off)};
            parts.push_back({off + 4, size});
            off += 8 + size;
            if (lead >= 0) break;
        }
        if (parts.size() == 1) {
            spans.push_back(parts[0]);
            joined_idx.push_back(-1);
        } else {
            std::vector<unsigned char> j;
            for (auto &p : parts) j.insert(j.end(), r.data.begin() + p.first, r.data.begin() + p.first + p.second);
            joined_idx.push_back((int)r.joined.size());
            r.joined.push_back(std::move(j));
            spans.push_back({0, 0});
        }
    }
    for (size_t k = 0; k < spans.size(); k++) {
        if (joined_idx[k] >= 0) {
            r.ptr.push_back(r.joined[joined_idx[k]].data());
            r.len.push_back(r.joined[joined_idx[k]].size());
        } else {
            r.ptr.push_back(r.data.data() + spans[k].first);
            r.len.push_back(spans[k].second);
        }
    }
    return r;
}

// read_mrconee.F90:1-222: 64-bit integers when record 3 is 8 + 4 * 2n bytes and record 4 is
// 8 (2n)^2 bytes for the n that record 3 starts with.
bool detect_32bit(const Records &r) {
    if (r.ptr.size() < 4) return true;
    if (r.len[2] >= 8) {
        const int64_t ns = rd_i64(r.ptr[2]);
        if (ns > 0 && ns < 10000 && r.len[2] == (size_t)(8 + 4 * 2 * ns) && r.len[3] == (size_t)(8 * (2 * ns) * (2 * ns)))
            return false;
    }
    return true;
}

int64_t rd_int(const unsigned char *p, bool is32) { return is32 ? (int64_t)rd_i32(p) : rd_i64(p); }

// read_mrconee.F90:602-715: energy order -> inactive, RAS1, RAS2, RAS3, secondary order.
// Inactive and secondary are the energy-ordered spinors in no RAS list, in order.
std::vector<double> ras_order(const std::vector<double> &e_sorted, const dcg_active_input &inp) {
    if (inp.nras1 == 0 && inp.nras2 == 0 && inp.nras3 == 0) return e_sorted;
    const int nmo = (int)e_sorted.size();
    std::set<int> in_ras;
    const int32_t *lists[3] = {inp.ras1, inp.ras2, inp.ras3};
    const int nl[3] = {inp.nras1, inp.nras2, inp.nras3};
    for (int l = 0; l < 3; l++)
        for (int q = 0; q < nl[l]; q++) {
            const int e = lists[l][q];
            if (e < 1 || e > nmo) throw IoError{DCG_E_ARG, "RAS list entry " + std::to_string(e) + " outside 1..nmo"};
            in_ras.insert(e);
        }
    std::vector<int> rest;
    for (int e = 1; e <= nmo; e++)
        if (!in_ras.count(e)) rest.push_back(e);
    std::vector<double> out = e_sorted;
    size_t k = 0;
    int pos = 0;
    for (; pos < inp.ninact; pos++) {
        if (k >= rest.size()) throw IoError{DCG_E_ARG, "RAS: not enough spinors outside the lists"};
        out[pos] = e_sorted[rest[k++] - 1];
    }
    for (int l = 0; l < 3; l++)
        for (int q = 0; q < nl[l]; q++) out[pos++] = e_sorted[lists[l][q] - 1];
    if (pos != inp.ninact + inp.nact) throw IoError{DCG_E_ARG, "RAS lists do not fill the active space"};
    for (; pos < inp.ninact + inp.nact + inp.nsec && pos < nmo; pos++) {
        if (k >= rest.size()) throw IoError{DCG_E_ARG, "RAS: not enough spinors outside the lists"};
        out[pos] = e_sorted[rest[k++] - 1];
    }
    return out;
}

template <typename T>
T *cnew(size_t n) {
    T *p = (T *)std::calloc(n ? n : 1, sizeof(T));
    if (!p) throw IoError{DCG_E_IO, "host allocation failed"};
    return p;
}

dcg_mrconee *read_mrconee(const std::string &path, const dcg_active_input &inp) {
    const Records r = read_records(path);
    if (r.ptr.size() < 6) throw IoError{DCG_E_IO, path + ": fewer than 6 records"};
    const bool is32 = detect_32bit(r);
    const size_t isz = is32 ? 4 : 8;
    // record 1: NMO, BREIT, ECORE, nfsym, nz, spinfr, norbt, hf_energy
    if (r.len[0] < 2 * isz + 8) throw IoError{DCG_E_IO, path + ": record 1 too short"};
    const int64_t nmo64 = rd_int(r.ptr[0], is32);
    if (nmo64 <= 0 || nmo64 > 1000000) throw IoError{DCG_E_IO, path + ": implausible NMO"};
    const int nmo = (int)nmo64;
    size_t off = 2 * isz;
    const double ecore = rd_f64(r.ptr[0] + off);
    off += 8 + 4 * isz;
    const double hf = r.len[0] >= off + 8 ? rd_f64(r.ptr[0] + off) : 0.0;
    // record 3: NSYMRPA, REPNA(2n); record 4: MULTB(2n, 2n)
    const int64_t ns = rd_int(r.ptr[2], is32);
    if (ns <= 0 || ns > 1024) throw IoError{DCG_E_IO, path + ": implausible NSYMRPA"};
    const int n2 = (int)(2 * ns);
    if (r.len[3] < (size_t)n2 * n2 * isz) throw IoError{DCG_E_IO, path + ": MULTB record too short"};
    // record 5: (IRPMO, IRPAMO, ORBMO) per spinor
    const size_t stride5 = 2 * isz + 8;
    if (r.len[4] < (size_t)nmo * stride5) throw IoError{DCG_E_IO, path + ": orbital record too short"};
    if (r.len[5] < (size_t)nmo * nmo * 16) throw IoError{DCG_E_IO, path + ": one-electron record too short"};
    if (inp.ninact + inp.nact + inp.nsec > nmo) throw IoError{DCG_E_ARG, "ninact + nact + nsec exceeds NMO"};

    dcg_mrconee *m = cnew<dcg_mrconee>(1);
    m->nmo = nmo;
    m->nsymrpa = (int32_t)ns;
    m->dirac_32bit = is32 ? 1 : 0;
    m->ecore = ecore;
    m->hf_energy = hf;
    m->multb = cnew<int32_t>((size_t)n2 * n2);
    for (int q = 0; q < n2 * n2; q++) m->multb[q] = (int32_t)rd_int(r.ptr[3] + q * isz, is32);   // file order = column-major
    std::vector<int64_t> irp_dirac(nmo);
    std::vector<double> e_dirac(nmo);
    for (int i = 0; i < nmo; i++) {
        irp_dirac[i] = rd_int(r.ptr[4] + i * stride5 + isz, is32);
        e_dirac[i] = rd_f64(r.ptr[4] + i * stride5 + 2 * isz);
    }
    std::vector<double> e_sorted = e_dirac;
    std::sort(e_sorted.begin(), e_sorted.end());
    const std::vector<double> e_cas = ras_order(e_sorted, inp);
    m->mo_energy = cnew<double>(nmo);
    std::copy(e_cas.begin(), e_cas.end(), m->mo_energy);
    // Kramers pairing: the first spinor of equal energy goes to i0, a later one to i0 + 1
    m->dirac_to_cas = cnew<int32_t>((size_t)nmo + 1);
    m->cas_to_dirac = cnew<int32_t>((size_t)nmo + 1);
    for (int i0 = 1; i0 <= nmo; i0 += 2) {
        int cnt = 0;
        for (int j0 = 1; j0 <= nmo; j0++) {
            if (e_dirac[j0 - 1] != e_cas[i0 - 1]) continue;
            if (cnt == 0) {
                m->cas_to_dirac[i0] = j0;
                m->dirac_to_cas[j0] = i0;
                cnt++;
            } else if (i0 + 1 <= nmo) {
                m->cas_to_dirac[i0 + 1] = j0;
                m->dirac_to_cas[j0] = i0 + 1;
            }
        }
    }
    for (int i = 1; i <= nmo; i++)
        if (m->cas_to_dirac[i] == 0) {
            dcg_free_mrconee(m);
            throw IoError{DCG_E_IO, path + ": Kramers pairing by equal orbital energy failed"};
        }
    m->irpamo = cnew<int32_t>(nmo);
    for (int i = 0; i < nmo; i++) m->irpamo[i] = (int32_t)irp_dirac[m->cas_to_dirac[i + 1] - 1];
    // record 6: ((ONER(i,j), ONEI(i,j), j = 1..nmo), i = 1..nmo); Im flipped from DIRAC 21
    m->h_re = cnew<double>((size_t)nmo * nmo);
    m->h_im = cnew<double>((size_t)nmo * nmo);
    const double sgn = inp.diracver >= 21 ? -1.0 : 1.0;
    for (int i0 = 0; i0 < nmo; i0++)
        for (int j0 = 0; j0 < nmo; j0++) {
            const unsigned char *p = r.ptr[5] + 16 * ((size_t)i0 * nmo + j0);
            const size_t ic = (size_t)m->dirac_to_cas[i0 + 1] - 1, jc = (size_t)m->dirac_to_cas[j0 + 1] - 1;
            m->h_re[ic + (size_t)nmo * jc] = rd_f64(p);
            m->h_im[ic + (size_t)nmo * jc] = sgn * rd_f64(p + 8);
        }
    return m;
}

bool file_exists(const std::string &p) {
    FILE *f = std::fopen(p.c_str(), "rb");
    if (!f) return false;
    std::fclose(f);
    return true;
}

// dcg_mdcint_raw followed by its storage; the caller sees only the first member.
struct MdcintOwned {
    dcg_mdcint_raw raw;
    int64_t *rec_off;
    int32_t *ikr, *jkr, *indk, *indl, *kr, *d2c;
    double *re, *im;
    int pinned;
};

void free_entries(MdcintOwned *o) {
    void *arr[4] = {o->indk, o->indl, o->re, o->im};
    for (void *p : arr) {
        if (!p) continue;
        if (o->pinned) cudaFreeHost(p);
        else std::free(p);
    }
}

template <typename T>
T *entry_alloc(size_t n, bool pinned) {
    if (!pinned) return cnew<T>(n);
    void *p = nullptr;
    const cudaError_t e = cudaHostAlloc(&p, (n ? n : 1) * sizeof(T), cudaHostAllocDefault);
    if (e != cudaSuccess) throw IoError{DCG_E_IO, std::string("page-locked allocation failed: ") + cudaGetErrorString(e)};
    return (T *)p;
}

dcg_mdcint_raw *read_mdcint(const std::string &dir, const dcg_mrconee &mrc, const dcg_active_input &inp, bool pinned) {
    std::vector<std::string> files{dir + "/MDCINT"};
    for (int k = 1;; k++) {
        const std::string p = dir + "/MDCINXXXX" + std::to_string(k);
        if (!file_exists(p)) break;
        files.push_back(p);
    }
    const bool is32 = mrc.dirac_32bit != 0;
    const size_t isz = is32 ? 4 : 8;
    // first pass: record table of every file
    std::vector<Records> recs;
    for (const std::string &f : files) recs.push_back(read_records(f));
    if (recs[0].ptr.empty()) throw IoError{DCG_E_IO, files[0] + ": empty"};
    const unsigned char *hdr = recs[0].ptr[0];
    if (recs[0].len[0] < 18 + isz) throw IoError{DCG_E_IO, files[0] + ": header too short"};
    const int64_t nkr = rd_int(hdr + 18, is32);
    if (nkr < 0 || recs[0].len[0] < 18 + isz + 2 * (size_t)nkr * isz) throw IoError{DCG_E_IO, files[0] + ": bad header"};
    int realonly = -1;
    struct Rec {
        const unsigned char *p;
        int64_t ikr, jkr, nz;
    };
    std::vector<Rec> all;
    int64_t nent = 0;
    for (size_t fi = 0; fi < recs.size(); fi++) {
        const Records &R = recs[fi];
        for (size_t k = 1; k < R.ptr.size(); k++) {   // record 0 of every file is its header
            if (R.len[k] < isz) continue;
            const int64_t ikr = rd_int(R.ptr[k], is32);
            if (ikr == 0) break;
            if (R.len[k] < 3 * isz) throw IoError{DCG_E_IO, files[fi] + ": record too short"};
            const int64_t jkr = rd_int(R.ptr[k] + isz, is32);
            const int64_t nz = rd_int(R.ptr[k] + 2 * isz, is32);
            if (nz <= 0) continue;
            const size_t voff = 3 * isz + 2 * (size_t)nz * isz;
            if (realonly < 0) realonly = R.len[k] < voff + 16 * (size_t)nz ? 1 : 0;
            if (R.len[k] < voff + (realonly ? 8 : 16) * (size_t)nz) throw IoError{DCG_E_IO, files[fi] + ": record too short"};
            all.push_back({R.ptr[k], ikr, jkr, nz});
            nent += nz;
        }
    }
    if (realonly < 0) realonly = 1;

    MdcintOwned *o = cnew<MdcintOwned>(1);
    o->pinned = pinned ? 1 : 0;
    try {
        const size_t nrec = all.size();
        o->rec_off = cnew<int64_t>(nrec + 1);
        o->ikr = cnew<int32_t>(nrec);
        o->jkr = cnew<int32_t>(nrec);
        o->kr = cnew<int32_t>(2 * (size_t)nkr);
        o->d2c = cnew<int32_t>((size_t)mrc.nmo + 1);
        o->indk = entry_alloc<int32_t>(nent, pinned);
        o->indl = entry_alloc<int32_t>(nent, pinned);
        o->re = entry_alloc<double>(nent, pinned);
        o->im = realonly ? nullptr : entry_alloc<double>(nent, pinned);
        for (int64_t q = 0; q < 2 * nkr; q++) o->kr[q] = (int32_t)rd_int(hdr + 18 + isz + q * isz, is32);
        for (int i = 0; i <= mrc.nmo; i++) o->d2c[i] = mrc.dirac_to_cas[i];
        int64_t e = 0;
        for (size_t r = 0; r < nrec; r++) {
            const Rec &R = all[r];
            o->rec_off[r] = e;
            o->ikr[r] = (int32_t)R.ikr;
            o->jkr[r] = (int32_t)R.jkr;
            const unsigned char *ind = R.p + 3 * isz;
            const unsigned char *val = ind + 2 * (size_t)R.nz * isz;
            for (int64_t n = 0; n < R.nz; n++) {
                o->indk[e + n] = (int32_t)rd_int(ind + (2 * n) * isz, is32);
                o->indl[e + n] = (int32_t)rd_int(ind + (2 * n + 1) * isz, is32);
                if (realonly) {
                    o->re[e + n] = rd_f64(val + 8 * n);
                } else {
                    o->re[e + n] = rd_f64(val + 16 * n);
                    o->im[e + n] = rd_f64(val + 16 * n + 8);
                }
            }
            e += R.nz;
        }
        o->rec_off[nrec] = e;
        dcg_mdcint_raw &w = o->raw;
        w.nrec = (int64_t)nrec;
        w.nent = nent;
        w.rec_off = o->rec_off;
        w.ikr = o->ikr;
        w.jkr = o->jkr;
        w.indk = o->indk;
        w.indl = o->indl;
        w.re = o->re;
        w.im = o->im;
        w.nkr = (int32_t)nkr;
        w.kr = o->kr;
        w.nmo = mrc.nmo;
        w.dirac_to_cas = o->d2c;
        w.scheme = inp.scheme ? inp.scheme : (inp.diracver > 22 ? 4 : 6);
        w.realonly = realonly;
    } catch (...) {
        dcg_free_mdcint(&o->raw);
        throw;
    }
    return &o->raw;
}

template <typename F>
int io_body(F &&f) {
    try {
        g_io_error.clear();
        f();
        return DCG_OK;
    } catch (const IoError &e) {
        g_io_error = e.msg;
        return e.code;
    } catch (const std::exception &e) {
        g_io_error = e.what();
        return DCG_E_IO;
    }
}

}  // namespace

extern "C" {

int dcg_read_mrconee(const char *path, const dcg_active_input *inp, dcg_mrconee **out) {
    if (!path || !inp || !out) {
        g_io_error = "null argument";
        return DCG_E_ARG;
    }
    *out = nullptr;
    return io_body([&] { *out = read_mrconee(path, *inp); });
}

void dcg_free_mrconee(dcg_mrconee *m) {
    if (!m) return;
    std::free(m->multb);
    std::free(m->irpamo);
    std::free(m->mo_energy);
    std::free(m->dirac_to_cas);
    std::free(m->cas_to_dirac);
    std::free(m->h_re);
    std::free(m->h_im);
    std::free(m);
}

int dcg_read_mdcint(const char *directory, const dcg_mrconee *mrc, const dcg_active_input *inp, int32_t pinned,
                    dcg_mdcint_raw **out) {
    if (!directory || !mrc || !inp || !out) {
        g_io_error = "null argument";
        return DCG_E_ARG;
    }
    *out = nullptr;
    return io_body([&] { *out = read_mdcint(directory, *mrc, *inp, pinned != 0); });
}

void dcg_free_mdcint(dcg_mdcint_raw *raw) {
    if (!raw) return;
    MdcintOwned *o = reinterpret_cast<MdcintOwned *>(raw);   // raw is the first member
    free_entries(o);
    std::free(o->rec_off);
    std::free(o->ikr);
    std::free(o->jkr);
    std::free(o->kr);
    std::free(o->d2c);
    std::free(o);
}

const char *dcg_io_last_error(void) { return g_io_error.c_str(); }

}  // extern "C"
