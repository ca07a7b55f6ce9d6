"""DIRAC file formats used by the CASPT2 hot path: ``active.inp``, ``MRCONEE`` and
``MDCINT``/``MDCINXXXX*`` (Fortran sequential unformatted), and the in-memory
MDCINTNEW record stream that the reference's ``create_newmdcint`` produces.

This is host-side input handling, not compute: it restates the reference readers
so that a caller without the Fortran driver can feed the C ABI.

Reference behaviour followed (paths within the reference project):
  * ``src/read_input_module.F90:50-240``  keyword parser (subset used here)
  * ``src/read_mrconee.F90:1-222``        32/64-bit DIRAC integer detection
  * ``src/read_mrconee.F90:226-600``      MRCONEE records, energy-order sort, Kramers pairing
  * ``src/read_mrconee.F90:602-715``      RAS reordering of the orbital list
  * ``src/module_realonly.F90:29-77``     real/complex MDCINT detection
  * ``src/create_newmdcint.F90:3-321``    MDCINT -> MDCINTNEW (scheme amplification,
                                          Kramers index map, canonical TYPE1-4 filter)
"""
from __future__ import annotations

import dataclasses
import os
import re
import struct
from typing import List, Optional, Tuple

import numpy as np

__all__ = [
    "ActiveInput", "MrconeeData", "MdcintNew",
    "read_active_inp", "read_fortran_records", "write_fortran_records",
    "read_mrconee", "read_mdcint_new", "mdcint_filenames", "Dfpcmo", "read_dfpcmo", "write_dfpcmo",
]


# --------------------------------------------------------------------------------------
# Fortran sequential unformatted records (gfortran layout, 4-byte markers, sub-records)
# --------------------------------------------------------------------------------------
def read_fortran_records(path: str) -> List[bytes]:
    """Return the payload of every record of a gfortran sequential unformatted file.

    A negative leading marker marks a continued sub-record (records > 2 GiB)."""
    data = open(path, "rb").read()
    out: List[bytes] = []
    off = 0
    n = len(data)
    while off < n:
        parts = []
        while True:
            if off + 4 > n:
                raise ValueError(f"{path}: truncated record marker at byte {off}")
            (lead,) = struct.unpack_from("<i", data, off)
            size = abs(lead)
            if off + 8 + size > n:
                raise ValueError(f"{path}: truncated record at byte {off}")
            parts.append(data[off + 4: off + 4 + size])
            off += 8 + size
            if lead >= 0:
                break
        out.append(b"".join(parts))
    return out


def write_fortran_records(path: str, records: List[bytes]) -> None:
    """Write records in gfortran sequential unformatted layout (sub-records above 2 GiB-1)."""
    limit = 2**31 - 9
    with open(path, "wb") as f:
        for rec in records:
            mv = memoryview(rec)
            if len(mv) == 0:
                f.write(struct.pack("<ii", 0, 0))
                continue
            pos = 0
            while pos < len(mv):
                chunk = mv[pos: pos + limit]
                last = pos + len(chunk) >= len(mv)
                marker = len(chunk) if last else -len(chunk)
                f.write(struct.pack("<i", marker))
                f.write(chunk)
                # gfortran: trailing marker of a continued sub-record is negative too
                f.write(struct.pack("<i", marker if last else -len(chunk)))
                pos += len(chunk)


# --------------------------------------------------------------------------------------
# active.inp
# --------------------------------------------------------------------------------------
@dataclasses.dataclass
class ActiveInput:
    ninact: int
    nact: int
    nsec: int
    nelec: int
    ciroots: List[Tuple[int, int]]          # (totsym, selectroot) pairs
    eshift: float = 0.0
    diracver: int = 21
    scheme: Optional[int] = None            # None -> default from diracver
    ras1: List[int] = dataclasses.field(default_factory=list)
    ras2: List[int] = dataclasses.field(default_factory=list)
    ras3: List[int] = dataclasses.field(default_factory=list)
    ras1_max_hole: int = 0
    ras3_max_elec: int = 0
    min_hole_ras1: int = 0
    min_elec_ras3: int = 0
    subprograms: Tuple[str, ...] = ("CASCI", "CASPT2")
    # IVO keywords (read_input_module.F90:150-201): .nhomo; .nocc/.nvcut without inversion
    # symmetry, .noccg/.noccu/.nvcutg/.nvcutu with it
    nhomo: int = 0
    occ_mo_num: Tuple[int, int] = (0, 0)
    vcut_mo_num: Tuple[int, int] = (0, 0)
    inversion: bool = False

    @property
    def mdcint_scheme(self) -> int:
        # read_input_module.F90:986-1011, module_global_variables.F90:44
        if self.scheme is not None:
            return self.scheme
        return 4 if self.diracver > 22 else 6

    @property
    def is_ras(self) -> bool:
        return bool(self.ras1 or self.ras2 or self.ras3)

    def to_text(self) -> str:
        lines = [".ninact", str(self.ninact), ".nact", str(self.nact), ".nsec", str(self.nsec),
                 ".nelec", str(self.nelec), ".caspt2_ciroots"]
        by_sym: dict = {}
        for s, r in self.ciroots:
            by_sym.setdefault(s, []).append(r)
        for s, rs in by_sym.items():
            lines.append(" ".join(str(x) for x in [s] + rs))
        lines += [".eshift", repr(float(self.eshift)), ".diracver", str(self.diracver)]
        if self.scheme is not None:
            lines += [".scheme", str(self.scheme)]
        if self.ras1:
            lines += [".ras1", _fmt_list(self.ras1), str(self.ras1_max_hole)]
        if self.ras2:
            lines += [".ras2", _fmt_list(self.ras2)]
        if self.ras3:
            lines += [".ras3", _fmt_list(self.ras3), str(self.ras3_max_elec)]
        if self.min_hole_ras1:
            lines += [".minholeras1", str(self.min_hole_ras1)]
        if self.min_elec_ras3:
            lines += [".minelecras3", str(self.min_elec_ras3)]
        lines += [".subprograms"] + list(self.subprograms) + [".end"]
        return "\n".join(lines) + "\n"


def _fmt_list(xs: List[int]) -> str:
    return ",".join(str(x) for x in xs)


def _parse_int_list(s: str) -> List[int]:
    """'3..4,9,11..12' -> [3,4,9,11,12] (read_input_module.F90 parse_input_string_to_int_list)."""
    out: List[int] = []
    for tok in re.split(r"[,\s]+", s.strip()):
        if not tok:
            continue
        if ".." in tok:
            a, b = tok.split("..")
            out.extend(range(int(a), int(b) + 1))
        else:
            out.append(int(tok))
    return sorted(out)


def read_active_inp(path_or_text: str) -> ActiveInput:
    """Parse the subset of ``active.inp`` keywords the CASCI/CASPT2 path consumes
    (read_input_module.F90:99-240)."""
    if os.path.exists(path_or_text):
        text = open(path_or_text).read()
    else:
        text = path_or_text
    raw = [ln.split("!")[0].split("#")[0].rstrip() for ln in text.splitlines()]
    lines = [ln.strip() for ln in raw if ln.strip()]
    kw: dict = {}
    i = 0
    ciroots: List[Tuple[int, int]] = []
    subprograms: List[str] = []
    while i < len(lines):
        key = lines[i].lower()
        i += 1
        if key == ".end":
            break
        if key == ".caspt2_ciroots":
            while i < len(lines) and not lines[i].startswith("."):
                nums = [int(x) for x in re.split(r"[\s,]+", lines[i].strip()) if x]
                sym = nums[0]
                for r in nums[1:]:
                    ciroots.append((sym, r))
                i += 1
        elif key == ".subprograms":
            while i < len(lines) and not lines[i].startswith("."):
                subprograms.append(lines[i].strip().upper())
                i += 1
        elif key in (".ras1", ".ras3"):
            kw[key] = _parse_int_list(lines[i])
            kw[key + "_max"] = int(lines[i + 1])
            i += 2
        elif key == ".ras2":
            kw[key] = _parse_int_list(lines[i])
            i += 1
        elif key in (".ninact", ".nact", ".nsec", ".nelec", ".diracver", ".scheme",
                     ".minholeras1", ".minelecras3", ".nhomo"):
            kw[key] = int(lines[i])
            i += 1
        elif key in (".nocc", ".nvcut", ".noccg", ".noccu", ".nvcutg", ".nvcutu"):
            inv = key in (".noccg", ".noccu", ".nvcutg", ".nvcutu")
            if kw.get("inversion", inv) != inv:
                raise ValueError("active.inp: .nocc/.nvcut and .noccg/.noccu/.nvcutg/.nvcutu exclude each other")
            kw["inversion"] = inv
            kw[key] = int(lines[i])
            i += 1
        elif key == ".eshift":
            kw[key] = float(lines[i].replace("d", "e").replace("D", "e"))
            i += 1
        else:
            # keywords outside the CASCI/CASPT2 path (IVO, restart, debug...) take one value line
            if i < len(lines) and not lines[i].startswith("."):
                i += 1
    for k in (".ninact", ".nact", ".nsec", ".nelec", ".diracver"):
        if k not in kw:
            raise ValueError(f"active.inp: essential keyword {k} missing")
    return ActiveInput(
        ninact=kw[".ninact"], nact=kw[".nact"], nsec=kw[".nsec"], nelec=kw[".nelec"],
        ciroots=ciroots, eshift=kw.get(".eshift", 0.0), diracver=kw[".diracver"],
        scheme=kw.get(".scheme"), ras1=kw.get(".ras1", []), ras2=kw.get(".ras2", []),
        ras3=kw.get(".ras3", []), ras1_max_hole=kw.get(".ras1_max", 0),
        ras3_max_elec=kw.get(".ras3_max", 0), min_hole_ras1=kw.get(".minholeras1", 0),
        min_elec_ras3=kw.get(".minelecras3", 0),
        subprograms=tuple(subprograms) if subprograms else ("CASCI", "CASPT2"),
        nhomo=kw.get(".nhomo", 0),
        occ_mo_num=(kw.get(".noccg", kw.get(".nocc", 0)), kw.get(".noccu", 0)),
        vcut_mo_num=(kw.get(".nvcutg", kw.get(".nvcut", 0)), kw.get(".nvcutu", 0)),
        inversion=bool(kw.get("inversion", False)))


# --------------------------------------------------------------------------------------
# MRCONEE
# --------------------------------------------------------------------------------------
@dataclasses.dataclass
class MrconeeData:
    nmo: int
    ecore: float
    nsymrpa: int
    repna: List[str]
    multb: np.ndarray            # (2n, 2n) int, 1-based values, Fortran (i0, j0) indexing at [i0-1, j0-1]
    irpamo: np.ndarray           # (nmo,) int, CAS (energy / RAS) order, 1-based irrep numbers
    mo_energy: np.ndarray        # (nmo,) CAS order (caspt2_mo_energy)
    dirac_to_cas: np.ndarray     # (nmo+1,) 1-based map, index 0 unused
    cas_to_dirac: np.ndarray     # (nmo+1,)
    h: np.ndarray                # (nmo, nmo) complex128 one-electron integrals in CAS order
    hf_energy: float
    dirac_32bit: bool

    @property
    def multb_s(self) -> np.ndarray:
        # read_mrconee.F90:417-419  MULTB_S = MULTB(n+1:2n, n+1:2n) - n
        n = self.nsymrpa
        return self.multb[n:2 * n, n:2 * n] - n

    @property
    def multb2(self) -> np.ndarray:
        # read_mrconee.F90:388-395  MULTB2(i0, MULTB(i0,j0)) = j0
        n2 = 2 * self.nsymrpa
        m2 = np.zeros((n2, n2), dtype=np.int64)
        for i0 in range(n2):
            for j0 in range(n2):
                m2[i0, self.multb[i0, j0] - 1] = j0 + 1
        return m2

    @property
    def multb_d(self) -> np.ndarray:
        # read_mrconee.F90:421  MULTB_D = MULTB2(1:n, 1:n) - n
        n = self.nsymrpa
        return self.multb2[0:n, 0:n] - n

    @property
    def multb_ds(self) -> np.ndarray:
        # read_mrconee.F90:429-440  MULTB_DS = transpose(MULTB(n+1:2n, 1:n))
        n = self.nsymrpa
        return np.ascontiguousarray(self.multb[n:2 * n, 0:n].T)


def _detect_dirac_32bit(recs: List[bytes]) -> bool:
    """read_mrconee.F90:1-222: 64-bit if record 3 has size 8 + 4*2*nsymrpa and record 4 8*(2n)^2."""
    r3 = recs[2]
    if len(r3) >= 8:
        nsymrpa = struct.unpack_from("<q", r3, 0)[0]
        if 0 < nsymrpa < 10000 and len(r3) == 8 + 4 * 2 * nsymrpa and len(recs[3]) == 8 * (2 * nsymrpa) ** 2:
            return False
    return True


def _ras_order(mo_sorted: np.ndarray, inp: ActiveInput) -> np.ndarray:
    """read_mrconee.F90:602-715: energy order -> (inactive, ras1, ras2, ras3, secondary) order."""
    ras1, ras2, ras3 = inp.ras1, inp.ras2, inp.ras3
    if not (ras1 or ras2 or ras3):
        return mo_sorted
    in_ras = set(ras1) | set(ras2) | set(ras3)
    out = mo_sorted.copy()
    nmo = len(mo_sorted)
    ninact, nact, nsec = inp.ninact, inp.nact, inp.nsec
    # inactive: first ninact energy-ordered spinors not in any RAS list
    rest = [e for e in range(1, nmo + 1) if e not in in_ras]
    k = 0
    for pos in range(ninact):
        out[pos] = mo_sorted[rest[k] - 1]
        k += 1
    pos = ninact
    for lst in (ras1, ras2, ras3):
        for e in lst:
            out[pos] = mo_sorted[e - 1]
            pos += 1
    if pos != ninact + nact:
        raise ValueError("RAS lists do not fill the active space")
    for pos in range(ninact + nact, ninact + nact + nsec):
        out[pos] = mo_sorted[rest[k] - 1]
        k += 1
    return out


def read_mrconee(path: str, inp: ActiveInput) -> MrconeeData:
    """Restatement of ``read_mrconee`` (read_mrconee.F90:226-600)."""
    recs = read_fortran_records(path)
    is32 = _detect_dirac_32bit(recs)
    it = "<i4" if is32 else "<i8"
    isz = 4 if is32 else 8
    r1 = recs[0]
    nmo = int(np.frombuffer(r1, it, 1, 0)[0])
    off = isz
    off += isz  # BREIT logical
    ecore = float(np.frombuffer(r1, "<f8", 1, off)[0]); off += 8
    off += isz * 2  # nfsym, nz
    off += isz      # spinfr
    off += isz      # norbt
    hf_energy = float(np.frombuffer(r1, "<f8", 1, off)[0])
    r3 = recs[2]
    nsymrpa = int(np.frombuffer(r3, it, 1, 0)[0])
    repna = [r3[isz + 4 * k: isz + 4 * (k + 1)].decode("latin-1") for k in range(2 * nsymrpa)]
    n2 = 2 * nsymrpa
    flat = np.frombuffer(recs[3], it, n2 * n2, 0).astype(np.int64)
    multb = flat.reshape(n2, n2).T.copy()          # Fortran column-major (i0 fastest)
    r5 = recs[4]
    dt = np.dtype([("irpmo", it), ("irpamo", it), ("e", "<f8")])
    mo = np.frombuffer(r5, dt, nmo, 0)
    irpamo_dirac = mo["irpamo"].astype(np.int64)
    e_dirac = mo["e"].astype(np.float64)
    # energy-order sort (heapSort ascending) then optional RAS order
    e_sorted = np.sort(e_dirac, kind="stable")
    e_cas = _ras_order(e_sorted, inp)
    # Kramers pairing by exact equal energies (read_mrconee.F90:515-530)
    cas_to_dirac = np.zeros(nmo + 1, dtype=np.int64)
    dirac_to_cas = np.zeros(nmo + 1, dtype=np.int64)
    for i0 in range(1, nmo + 1, 2):
        m = 0
        for j0 in range(1, nmo + 1):
            if e_dirac[j0 - 1] == e_cas[i0 - 1]:
                if m == 0:
                    cas_to_dirac[i0] = j0
                    dirac_to_cas[j0] = i0
                    m += 1
                else:
                    cas_to_dirac[i0 + 1] = j0
                    dirac_to_cas[j0] = i0 + 1
    if np.any(cas_to_dirac[1:] == 0):
        raise ValueError("MRCONEE: Kramers pairing by equal orbital energy failed")
    irpamo = irpamo_dirac[cas_to_dirac[1:] - 1]
    # one-electron integrals ((ONER(i,j), ONEI(i,j), j=1..nmo), i=1..nmo)
    r6 = np.frombuffer(recs[5], "<f8", 2 * nmo * nmo, 0).reshape(nmo, nmo, 2)
    oner = r6[:, :, 0]   # [i, j] (j fastest)
    onei = r6[:, :, 1]
    if inp.diracver >= 21:
        onei = -onei     # read_mrconee.F90:579-581
    h = np.zeros((nmo, nmo), dtype=np.complex128)
    d2c = dirac_to_cas[1:] - 1
    h[np.ix_(d2c, d2c)] = oner + 1j * onei
    return MrconeeData(nmo=nmo, ecore=ecore, nsymrpa=nsymrpa, repna=repna, multb=multb,
                       irpamo=irpamo, mo_energy=e_cas, dirac_to_cas=dirac_to_cas,
                       cas_to_dirac=cas_to_dirac, h=h, hf_energy=hf_energy, dirac_32bit=is32)


# --------------------------------------------------------------------------------------
# MDCINT -> MDCINTNEW
# --------------------------------------------------------------------------------------
@dataclasses.dataclass
class MdcintNew:
    """MDCINTNEW records (create_newmdcint.F90:171-177) as structure-of-arrays.

    ``idx`` is (n, 4) int32 with 1-based CAS-order spinor indices (i, j, k, l) of (ij|kl);
    ``val`` the complex value exactly as written (Re, -Im of the DIRAC record)."""
    idx: np.ndarray
    val: np.ndarray
    realonly: bool

    def __len__(self) -> int:
        return int(self.idx.shape[0])


def mdcint_filenames(directory: str) -> List[str]:
    """MDCINT then MDCINXXXX1, MDCINXXXX2, ... while they exist (get_filename.F90:1-41)."""
    out = [os.path.join(directory, "MDCINT")]
    k = 1
    while True:
        p = os.path.join(directory, f"MDCINXXXX{k}")
        if not os.path.exists(p):
            break
        out.append(p)
        k += 1
    return out


def _parse_mdcint_file(recs: List[bytes], is32: bool, realonly: Optional[bool], skip_header: bool):
    it = np.dtype("<i4" if is32 else "<i8")
    isz = it.itemsize
    out = []
    start = 1 if skip_header else 0
    for rec in recs[start:]:
        if len(rec) < isz:
            continue
        ikr = int(np.frombuffer(rec, it, 1, 0)[0])
        if ikr == 0:
            break
        jkr = int(np.frombuffer(rec, it, 1, isz)[0])
        nz = int(np.frombuffer(rec, it, 1, 2 * isz)[0])
        if nz <= 0:
            continue
        ind = np.frombuffer(rec, it, 2 * nz, 3 * isz).astype(np.int64).reshape(nz, 2)
        voff = 3 * isz + 2 * nz * isz
        if realonly is None:
            realonly = len(rec) < voff + 16 * nz
        if realonly:
            vr = np.frombuffer(rec, "<f8", nz, voff).copy()
            vi = np.zeros(nz)
        else:
            v = np.frombuffer(rec, "<f8", 2 * nz, voff).reshape(nz, 2)
            vr = v[:, 0].copy()
            vi = v[:, 1].copy()
        out.append((ikr, jkr, ind[:, 0].copy(), ind[:, 1].copy(), vr, vi))
    return out, realonly


@dataclasses.dataclass
class MdcintRaw:
    """DIRAC's MDCINT records flattened in file order (the input of create_newmdcint and of
    the library's dcg_mdcint_canonicalize): per record the signed Kramers-pair indices
    (ikr, jkr) and the entry range rec_off[r]:rec_off[r+1]; per entry (indk, indl) and the
    stored value; the header's Kramers table and the DIRAC-to-CAS map."""
    rec_ikr: np.ndarray        # (nrec,) int32
    rec_jkr: np.ndarray        # (nrec,) int32
    rec_off: np.ndarray        # (nrec + 1,) int64
    indk: np.ndarray           # (nent,) int32
    indl: np.ndarray           # (nent,) int32
    re: np.ndarray             # (nent,) float64
    im: np.ndarray             # (nent,) float64 (zeros when real-only)
    kr: np.ndarray             # (nkr, 2) int32: kr(i), kr(-i)
    nmo: int
    dirac_to_cas: np.ndarray   # (nmo + 1,) int32, 1-based, [0] unused
    scheme: int
    realonly: bool


def read_mdcint_raw(directory: str, mrc: MrconeeData, inp: ActiveInput) -> MdcintRaw:
    """Every record of MDCINT, MDCINXXXX1, ... (create_newmdcint.F90:3-171's reads)."""
    files = mdcint_filenames(directory)
    is32 = mrc.dirac_32bit
    it = "<i4" if is32 else "<i8"
    isz = 4 if is32 else 8
    hdr = read_fortran_records(files[0])[0]
    nkr = int(np.frombuffer(hdr, it, 1, 18)[0])
    pairs = np.frombuffer(hdr, it, 2 * nkr, 18 + isz).astype(np.int64).reshape(nkr, 2)
    realonly: Optional[bool] = None
    ikr_l, jkr_l, nz_l, k_l, l_l, re_l, im_l = [], [], [], [], [], [], []
    for fname in files:
        recs = read_fortran_records(fname)
        if not recs:
            continue
        parsed, realonly = _parse_mdcint_file(recs, is32, realonly, skip_header=True)
        for (ikr0, jkr0, indk0, indl0, rr0, ri0) in parsed:
            ikr_l.append(ikr0)
            jkr_l.append(jkr0)
            nz_l.append(len(indk0))
            k_l.append(indk0)
            l_l.append(indl0)
            re_l.append(rr0)
            im_l.append(ri0)
    if realonly is None:
        realonly = True
    off = np.zeros(len(nz_l) + 1, dtype=np.int64)
    off[1:] = np.cumsum(nz_l) if nz_l else []
    cat = (lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt))
    return MdcintRaw(rec_ikr=np.array(ikr_l, np.int32), rec_jkr=np.array(jkr_l, np.int32), rec_off=off,
                     indk=cat(k_l, np.int32), indl=cat(l_l, np.int32), re=cat(re_l, np.float64),
                     im=cat(im_l, np.float64), kr=pairs.astype(np.int32), nmo=int(mrc.nmo),
                     dirac_to_cas=np.asarray(mrc.dirac_to_cas, np.int32), scheme=int(inp.mdcint_scheme),
                     realonly=bool(realonly))


def write_mdcint_raw(path: str, raw: MdcintRaw, is32: bool, realonly: Optional[bool] = None,
                     header_stamp: bytes = b" 01Jan26  00:00:00") -> None:
    """Write ``raw`` back as one DIRAC MDCINT file (the layout create_newmdcint.F90:210-265 and
    module_realonly.F90:29-77 read): header ``datex, timex, nkr, (kr(i), kr(-i))``, one record
    ``ikr, jkr, nz, (indk, indl) * nz, values`` per raw record, and the ``ikr = 0`` end record.
    The values are ``re`` alone (real-only layout) or interleaved ``(re, im)`` pairs (complex
    layout); ``realonly`` defaults to ``raw.realonly``, and a real-only ``raw`` written in the
    complex layout gets zero imaginary parts, which makes check_realonly report complex."""
    it = "<i4" if is32 else "<i8"
    ro = raw.realonly if realonly is None else bool(realonly)
    ints = lambda *xs: np.array(xs, it).tobytes()
    hdr = header_stamp[:18].ljust(18) + ints(len(raw.kr)) + np.asarray(raw.kr, it).reshape(-1).tobytes()
    recs = [hdr]
    for r in range(len(raw.rec_ikr)):
        a, b = int(raw.rec_off[r]), int(raw.rec_off[r + 1])
        kl = np.stack([raw.indk[a:b], raw.indl[a:b]], axis=1).astype(it).tobytes()
        if ro:
            vv = np.asarray(raw.re[a:b], "<f8").tobytes()
        else:
            vv = np.stack([raw.re[a:b], raw.im[a:b]], axis=1).astype("<f8").tobytes()
        recs.append(ints(int(raw.rec_ikr[r]), int(raw.rec_jkr[r]), b - a) + kl + vv)
    recs.append(ints(0, 0, 0))
    write_fortran_records(path, recs)


def canonicalize_mdcint(raw: MdcintRaw) -> MdcintNew:
    """Restatement of create_newmdcint's canonicalisation (create_newmdcint.F90:171-321) on
    the raw records: both Kramers partners of every record, the bra/ket-exchanged copies of
    schemes other than 6, the TYPE1-4 filter, the 0.25e-12 cutoff, CAS order."""
    nkr = raw.kr.shape[0]
    kr = np.zeros(2 * nkr + 1, dtype=np.int64)   # kr(-nkr : nkr) stored at offset nkr
    o = nkr
    kr[o + np.arange(1, nkr + 1)] = raw.kr[:, 0]
    kr[o - np.arange(1, nkr + 1)] = raw.kr[:, 1]
    scheme = raw.scheme
    realonly = raw.realonly
    out_i, out_v = [], []
    cutoff = 0.25e-12
    d2c = raw.dirac_to_cas.astype(np.int64)
    for r in range(len(raw.rec_ikr)):
        a, b = int(raw.rec_off[r]), int(raw.rec_off[r + 1])
        nz = b - a
        if nz <= 0:
            continue
        ikr0, jkr0 = int(raw.rec_ikr[r]), int(raw.rec_jkr[r])
        indk0 = raw.indk[a:b].astype(np.int64)
        indl0 = raw.indl[a:b].astype(np.int64)
        rr0, ri0 = raw.re[a:b], raw.im[a:b]
        ikr, jkr, indk, indl, rr, ri = ikr0, jkr0, indk0, indl0, rr0, ri0
        for n in (1, 2):
            if n == 2:
                ikr, jkr, indk, indl = -ikr, -jkr, -indk, -indl
                sgn = np.where(ikr * jkr * indk * indl >= 0, 1.0, -1.0)
                rr = -rr * sgn
                ri = ri * sgn
            amplify = (scheme != 6 and abs(ikr) != abs(jkr))
            reps = 2 if amplify else 1
            for rep in range(reps):
                ci = np.full(nz, ikr, dtype=np.int64)
                cj = np.full(nz, jkr, dtype=np.int64)
                ck = indk.copy()
                cl = indl.copy()
                vr = rr.copy()
                vi = ri.copy()
                if rep == 1:
                    ci, cj = cj, ci
                    ck, cl = cl, ck
                    t23 = (((ci < 0).astype(int) + (cj < 0).astype(int)) == 1) & \
                          (((ck < 0).astype(int) + (cl < 0).astype(int)) == 1)
                    ci = np.where(t23, -ci, ci)
                    cj = np.where(t23, -cj, cj)
                    ck = np.where(t23, -ck, ck)
                    cl = np.where(t23, -cl, cl)
                    if not realonly:
                        vi = np.where(t23, vi, -vi)
                iii = d2c[kr[o + ci]]
                jjj = d2c[kr[o + cj]]
                kkk = d2c[kr[o + ck]]
                lll = d2c[kr[o + cl]]

                def kr_signed(x):
                    return np.where(x % 2 == 1, 1, -1) * (x // 2 + x % 2)

                ikk, jkk, kkk_, lkk = kr_signed(iii), kr_signed(jjj), kr_signed(kkk), kr_signed(lll)
                ii, jj, kk, ll = np.abs(ikk), np.abs(jkk), np.abs(kkk_), np.abs(lkk)
                if realonly:
                    big = np.abs(rr) > cutoff
                else:
                    big = (np.abs(rr) > cutoff) | (np.abs(ri) > cutoff)
                t1 = (ikk > 0) & (jkk > 0) & (kkk_ > 0) & (lkk > 0)
                t2 = (ikk > 0) & (jkk < 0) & (kkk_ > 0) & (lkk < 0)
                t3 = (ikk > 0) & (jkk < 0) & (kkk_ < 0) & (lkk > 0)
                t4 = (ikk > 0) & (jkk < 0) & (kkk_ < 0) & (lkk < 0)
                c1 = ((ii <= jj) & (kk <= ll) & ((ii < kk) | ((ii == kk) & (jj <= ll)))) | \
                     ((ii <= jj) & (ll <= kk) & ((ii < ll) | ((ii == ll) & (jj <= kk))))
                c23 = (ii <= jj) & (kk <= ll) & ((ii < kk) | ((ii == kk) & (jj <= ll)))
                c4 = ii <= jj
                keep = big & ((t1 & c1) | (t2 & c23) | (t3 & c23) | (t4 & c4))
                if not np.any(keep):
                    continue

                def swapkr(x):
                    return np.where(x % 2 == 1, x + 1, x - 1)

                q = np.stack([swapkr(iii), swapkr(jjj), swapkr(kkk), swapkr(lll)], axis=1)[keep]
                out_i.append(q.astype(np.int32))
                out_v.append((vr - 1j * vi)[keep] if not realonly else vr[keep] + 0j)
    idx = np.concatenate(out_i) if out_i else np.zeros((0, 4), np.int32)
    val = np.concatenate(out_v) if out_v else np.zeros(0, np.complex128)
    return MdcintNew(idx=idx, val=val, realonly=bool(realonly))


def read_mdcint_new(directory: str, mrc: MrconeeData, inp: ActiveInput) -> MdcintNew:
    """Restatement of ``create_newmdcint`` (create_newmdcint.F90:3-321) returning the
    MDCINTNEW records in memory instead of on disk."""
    return canonicalize_mdcint(read_mdcint_raw(directory, mrc, inp))


# --------------------------------------------------------------------------------------
# DFPCMO (DIRAC's formatted MO coefficient file; read and rewritten by the IVO program)
# --------------------------------------------------------------------------------------
@dataclasses.dataclass
class Dfpcmo:
    """DFPCMO as fockivo.F90:87-160 reads it.  With DIRAC >= 21 the sections carry title
    lines (INFO, COEFS, EVALS, SUPERSYM, KAPPA), kept verbatim; ``nfsym`` is the number of
    fermion-irrep groups (2 with inversion symmetry), ``nfsym2`` the second integer of the
    dimension line of the new format."""
    titles: dict                 # "info", "coefs", "evals", "supersym", "kappa" -> line or None
    name_line: str
    energy_line: str
    nfsym: int
    nfsym2: Optional[int]
    positronic: List[int]
    electronic: List[int]
    basis_ao: List[int]
    coef: np.ndarray             # (total_ao,) float64, per group MO-major blocks
    evals: np.ndarray            # (total_mo,)
    supersym: np.ndarray         # (total_mo,) int
    kappa: Optional[np.ndarray]  # (total_mo,) int or None
    new_format: bool

    @property
    def total_mo(self) -> int:
        return sum(self.positronic) + sum(self.electronic)

    @property
    def basis_all(self) -> List[int]:
        return [(p + e) * b for p, e, b in zip(self.positronic, self.electronic, self.basis_ao)]


def _tokens(lines: List[str], pos: int, n: int, conv):
    out = []
    while len(out) < n:
        if pos >= len(lines):
            raise ValueError("DFPCMO: unexpected end of file")
        out.extend(conv(t.replace("D", "E").replace("d", "e")) for t in lines[pos].split())
        pos += 1
    if len(out) != n:
        raise ValueError("DFPCMO: a list does not end on a line boundary")
    return out, pos


def read_dfpcmo(path: str, new_format: bool) -> Dfpcmo:
    """fockivo.F90:87-160 (list-directed reads; the title lines only with ``new_format``,
    i.e. DIRAC >= 21)."""
    lines = open(path).read().split("\n")
    if lines and lines[-1] == "":
        lines.pop()
    pos = 0
    titles = {}

    def title(key):
        nonlocal pos
        if new_format:
            titles[key] = lines[pos]
            pos += 1
        else:
            titles[key] = None

    title("info")
    name_line = lines[pos]
    pos += 1
    dims = [int(t) for t in lines[pos].split()]
    pos += 1
    nfsym = dims[0]
    rest = dims[2:] if new_format else dims[1:]
    nfsym2 = dims[1] if new_format else None
    positronic = [rest[3 * g] for g in range(nfsym)]
    electronic = [rest[3 * g + 1] for g in range(nfsym)]
    basis_ao = [rest[3 * g + 2] for g in range(nfsym)]
    energy_line = lines[pos]
    pos += 1
    title("coefs")
    total_ao = sum((p + e) * b for p, e, b in zip(positronic, electronic, basis_ao))
    total_mo = sum(positronic) + sum(electronic)
    coef, pos = _tokens(lines, pos, total_ao, float)
    title("evals")
    evals, pos = _tokens(lines, pos, total_mo, float)
    title("supersym")
    sup, pos = _tokens(lines, pos, total_mo, int)
    kappa = None
    while pos < len(lines) and not lines[pos].strip():
        pos += 1
    if pos < len(lines):
        title("kappa")
        kappa, pos = _tokens(lines, pos, total_mo, int)
        kappa = np.array(kappa, np.int64)
    else:
        titles["kappa"] = None
    return Dfpcmo(titles=titles, name_line=name_line, energy_line=energy_line, nfsym=nfsym, nfsym2=nfsym2,
                  positronic=positronic, electronic=electronic, basis_ao=basis_ao, coef=np.array(coef, np.float64),
                  evals=np.array(evals, np.float64), supersym=np.array(sup, np.int64), kappa=kappa,
                  new_format=new_format)


def _fortran_e(x: float, w: int = 22, d: int = 12) -> str:
    """Fortran Ew.d: 0.ddd...E+xx."""
    if x == 0.0:
        body = "0." + "0" * d + "E+00"
    else:
        m = f"{abs(x):.{d - 1}e}"
        digits = m[0] + m[2:2 + d - 1]
        ex = int(m.split("e")[1]) + 1
        body = ("-" if x < 0 else "") + "0." + digits + (f"E{ex:+03d}" if abs(ex) < 100 else f"{ex:+04d}")
    return body.rjust(w)


def _rows(items: List[str], per: int) -> List[str]:
    return ["".join(items[k:k + per]) for k in range(0, len(items), per)] or [""]


def write_dfpcmo(path: str, d: Dfpcmo) -> None:
    """fockivo.F90:296-346: the title lines as read (A150), the dimension line in I0 fields,
    coefficients 6F22.16, energies 6E22.12, supersymmetry and kappa 66(X,I0)."""
    out = []
    a150 = lambda s: s[:150].ljust(150)
    if d.new_format:
        out.append(a150(d.titles["info"]))
    out.append(a150(d.name_line))
    dims = [d.nfsym] + ([d.nfsym2] if d.new_format else [])
    for g in range(d.nfsym):
        dims += [d.positronic[g], d.electronic[g], d.basis_ao[g]]
    out.append("".join(f" {v}" for v in dims))
    out.append(a150(d.energy_line))
    if d.new_format:
        out.append(a150(d.titles["coefs"]))
    out += _rows([f"{x:22.16f}" for x in d.coef], 6)
    if d.new_format:
        out.append(a150(d.titles["evals"]))
    out += _rows([_fortran_e(float(x)) for x in d.evals], 6)
    if d.new_format:
        out.append(a150(d.titles["supersym"]))
    out += _rows([f" {int(v)}" for v in d.supersym], 66)
    if d.kappa is not None:
        if d.new_format:
            out.append(a150(d.titles["kappa"]))
        out += _rows([f" {int(v)}" for v in d.kappa], 66)
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
