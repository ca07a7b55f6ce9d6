"""Host-side mirror of the reference's CASCI/CASPT2 drivers over the C ABI.

``Caspt2Session`` wraps one library context (one CUDA stream on one GPU):

    set_system(system)  -> readint2_casci / divide_2_elec_integral_into_subspaces
    casci(nroot)        -> casci            (src/casci.F90:3-163)
    caspt2(skip_mask)   -> r4dcaspt2_tra    (src/r4dcaspt2_tra.F90:4-482)

``run_case(directory)`` is the whole reference flow for one ``.caspt2_ciroots`` entry
(src/dcaspt2_run_subprograms.F90:39-64) with the reference's printed energy lines.

The compute path is the CUDA library ``libdcaspt2_gb300.so``; there is no CPU fallback:
if the library is missing or no GPU is present, the calls raise.
"""
from __future__ import annotations

import ctypes
import dataclasses
import os
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libdcaspt2_gb300.so")

DCG_PREC_FP64 = 0
DCG_PREC_SPLIT = 1
DCG_PREC_SPLIT_ACC = 2   # dcg_zgemm: the seven-slice split product
CASCI_SOLVERS = {"auto": 0, "dense": 1, "davidson": 2}
METRIC_SOLVERS = {"auto": 0, "eigen": 1}
SUBSPACES = "ABCDEFGH"
STAGES = ["ints", "casci_matrix", "casci_eig", "fock", "ci_rotation", "rdm", "transformation",
          "A", "B", "C", "D", "E", "F", "G", "H", "AC", "BDEFG"]


class DcgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"dcaspt2_gb300 error {code}: {msg}")
        self.code = code


class _System(ctypes.Structure):
    _fields_ = [
        ("ninact", ctypes.c_int32), ("nact", ctypes.c_int32), ("nsec", ctypes.c_int32), ("nelec", ctypes.c_int32),
        ("nmo", ctypes.c_int32), ("nsymrpa", ctypes.c_int32), ("totsym", ctypes.c_int32),
        ("selectroot", ctypes.c_int32), ("realonly", ctypes.c_int32), ("eshift", ctypes.c_double),
        ("ecore", ctypes.c_double), ("multb", ctypes.POINTER(ctypes.c_int32)),
        ("irpamo", ctypes.POINTER(ctypes.c_int32)), ("h_re", ctypes.POINTER(ctypes.c_double)),
        ("h_im", ctypes.POINTER(ctypes.c_double)), ("nrec", ctypes.c_int64),
        ("rec_ijkl", ctypes.POINTER(ctypes.c_int32)), ("rec_re", ctypes.POINTER(ctypes.c_double)),
        ("rec_im", ctypes.POINTER(ctypes.c_double)),
        ("ras1_size", ctypes.c_int32), ("ras2_size", ctypes.c_int32), ("ras3_size", ctypes.c_int32),
        ("ras1_max_hole", ctypes.c_int32), ("ras3_max_elec", ctypes.c_int32),
        ("min_hole_ras1", ctypes.c_int32), ("min_elec_ras3", ctypes.c_int32),
        ("rec_on_device", ctypes.c_int32),
    ]


class _MdcintRaw(ctypes.Structure):
    """dcg_mdcint_raw."""
    _fields_ = [
        ("nrec", ctypes.c_int64), ("nent", ctypes.c_int64), ("rec_off", ctypes.c_void_p),
        ("ikr", ctypes.c_void_p), ("jkr", ctypes.c_void_p), ("indk", ctypes.c_void_p), ("indl", ctypes.c_void_p),
        ("re", ctypes.c_void_p), ("im", ctypes.c_void_p), ("nkr", ctypes.c_int32), ("kr", ctypes.c_void_p),
        ("nmo", ctypes.c_int32), ("dirac_to_cas", ctypes.c_void_p), ("scheme", ctypes.c_int32),
        ("realonly", ctypes.c_int32),
    ]


class MdcintBuffers:
    """A dirac_io.MdcintRaw in the exact layout of dcg_mdcint_raw (arrays kept alive)."""

    def __init__(self, raw):
        self.arrays = dict(
            rec_off=np.ascontiguousarray(raw.rec_off, np.int64), ikr=np.ascontiguousarray(raw.rec_ikr, np.int32),
            jkr=np.ascontiguousarray(raw.rec_jkr, np.int32), indk=np.ascontiguousarray(raw.indk, np.int32),
            indl=np.ascontiguousarray(raw.indl, np.int32), re=np.ascontiguousarray(raw.re, np.float64),
            im=np.ascontiguousarray(raw.im, np.float64), kr=np.ascontiguousarray(raw.kr, np.int32),
            d2c=np.ascontiguousarray(raw.dirac_to_cas, np.int32))
        a = self.arrays
        st = _MdcintRaw()
        st.nrec = len(a["ikr"])
        st.nent = len(a["re"])
        for f, k in (("rec_off", "rec_off"), ("ikr", "ikr"), ("jkr", "jkr"), ("indk", "indk"), ("indl", "indl"),
                     ("re", "re"), ("kr", "kr"), ("dirac_to_cas", "d2c")):
            setattr(st, f, a[k].ctypes.data)
        st.im = None if raw.realonly else a["im"].ctypes.data
        st.nkr = a["kr"].shape[0]
        st.nmo = int(raw.nmo)
        st.scheme = int(raw.scheme)
        st.realonly = int(bool(raw.realonly))
        self.struct = st
        self.realonly = bool(raw.realonly)


class _ActiveInput(ctypes.Structure):
    """dcg_active_input."""
    _fields_ = [
        ("ninact", ctypes.c_int32), ("nact", ctypes.c_int32), ("nsec", ctypes.c_int32), ("nelec", ctypes.c_int32),
        ("diracver", ctypes.c_int32), ("scheme", ctypes.c_int32), ("nras1", ctypes.c_int32),
        ("nras2", ctypes.c_int32), ("nras3", ctypes.c_int32), ("ras1", ctypes.c_void_p), ("ras2", ctypes.c_void_p),
        ("ras3", ctypes.c_void_p),
    ]


class _Mrconee(ctypes.Structure):
    """dcg_mrconee."""
    _fields_ = [
        ("nmo", ctypes.c_int32), ("nsymrpa", ctypes.c_int32), ("dirac_32bit", ctypes.c_int32),
        ("ecore", ctypes.c_double), ("hf_energy", ctypes.c_double), ("multb", ctypes.POINTER(ctypes.c_int32)),
        ("irpamo", ctypes.POINTER(ctypes.c_int32)), ("mo_energy", ctypes.POINTER(ctypes.c_double)),
        ("dirac_to_cas", ctypes.POINTER(ctypes.c_int32)), ("cas_to_dirac", ctypes.POINTER(ctypes.c_int32)),
        ("h_re", ctypes.POINTER(ctypes.c_double)), ("h_im", ctypes.POINTER(ctypes.c_double)),
    ]


class _TuneEntry(ctypes.Structure):
    """dcg_tune_entry."""
    _fields_ = [("kind", ctypes.c_int32), ("ops", ctypes.c_int32), ("m", ctypes.c_int32), ("n", ctypes.c_int32),
                ("k", ctypes.c_int32), ("flags", ctypes.c_int32), ("choice", ctypes.c_int32),
                ("ncand", ctypes.c_int32), ("best_ms", ctypes.c_float), ("heuristic_ms", ctypes.c_float)]


class _RequestResult(ctypes.Structure):
    """dcg_request_result of the serving loop."""
    _fields_ = [
        ("request_id", ctypes.c_uint64), ("status", ctypes.c_int32), ("ndet", ctypes.c_int32),
        ("casci_energy", ctypes.c_double), ("e2", ctypes.c_double * 8), ("sumc2", ctypes.c_double * 8),
        ("e0", ctypes.c_double), ("etotal", ctypes.c_double), ("t_submit", ctypes.c_double),
        ("t_start", ctypes.c_double), ("t_end", ctypes.c_double), ("slot", ctypes.c_int32),
        ("attempts", ctypes.c_int32), ("error", ctypes.c_char * 96),
    ]


_lib = None


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    """Load the CUDA library (built by ``dirac_caspt2_gb300.build.build()``)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with dirac_caspt2_gb300.build.build() "
                          "(the CASPT2 path has no CPU fallback)")
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    lib.dcg_create.argtypes = [ctypes.c_int, ctypes.c_int, P(ctypes.c_void_p)]
    lib.dcg_destroy.argtypes = [ctypes.c_void_p]
    lib.dcg_last_error.argtypes = [ctypes.c_void_p]
    lib.dcg_last_error.restype = ctypes.c_char_p
    lib.dcg_set_system.argtypes = [ctypes.c_void_p, P(_System)]
    lib.dcg_casci.argtypes = [ctypes.c_void_p, ctypes.c_int32, P(ctypes.c_double), P(ctypes.c_double),
                              P(ctypes.c_double), P(ctypes.c_int32)]
    lib.dcg_caspt2.argtypes = [ctypes.c_void_p, ctypes.c_uint32, P(ctypes.c_double), P(ctypes.c_double),
                               P(ctypes.c_double), P(ctypes.c_double)]
    lib.dcg_get_eps.argtypes = [ctypes.c_void_p, P(ctypes.c_double), ctypes.c_int32]
    lib.dcg_caspt2_irreps.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p]
    lib.dcg_casci_determinants.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]
    lib.dcg_stage_times.argtypes = [ctypes.c_void_p, P(ctypes.c_double), ctypes.c_int32]
    lib.dcg_kernel_launches.argtypes = [ctypes.c_void_p]
    lib.dcg_kernel_launches.restype = ctypes.c_int64
    lib.dcg_version.restype = ctypes.c_char_p
    lib.dcg_solve_h.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                ctypes.c_int32, ctypes.c_double, P(ctypes.c_double)]
    lib.dcg_stream.argtypes = [ctypes.c_void_p]
    lib.dcg_stream.restype = ctypes.c_void_p
    lib.dcg_time_family.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    lib.dcg_set_wait_limit.argtypes = [ctypes.c_void_p, ctypes.c_double]
    lib.dcg_family_stats.argtypes = [ctypes.c_void_p, P(ctypes.c_double), P(ctypes.c_int64), P(ctypes.c_double)]
    lib.dcg_zgemm.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                              ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                              ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int64,
                              ctypes.c_int64, ctypes.c_int64, ctypes.c_int32]
    lib.dcg_stedc.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                              ctypes.c_void_p]
    lib.dcg_heev_batch.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.dcg_heev_range.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]
    lib.dcg_heev.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                             ctypes.c_void_p, ctypes.c_void_p]
    lib.dcg_mdcint_canonicalize.argtypes = [ctypes.c_void_p, P(_MdcintRaw), P(ctypes.c_int64)]
    lib.dcg_mdcint_records.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.dcg_set_system_mdcint.argtypes = [ctypes.c_void_p, P(_System), P(_MdcintRaw)]
    lib.dcg_set_casci_solver.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    lib.dcg_casci_iterations.argtypes = [ctypes.c_void_p]
    lib.dcg_casci_iterations.restype = ctypes.c_int32
    lib.dcg_set_metric_solver.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    lib.dcg_gram_cholesky_blocks.argtypes = [ctypes.c_void_p]
    lib.dcg_gram_cholesky_blocks.restype = ctypes.c_int32
    lib.dcg_gram_deflated_blocks.argtypes = [ctypes.c_void_p]
    lib.dcg_gram_deflated_blocks.restype = ctypes.c_int32
    lib.dcg_device_bytes.argtypes = [ctypes.c_void_p]
    lib.dcg_device_bytes.restype = ctypes.c_int64
    lib.dcg_trim.argtypes = [ctypes.c_void_p]
    lib.dcg_footprint_estimate.argtypes = [P(_System)]
    lib.dcg_footprint_estimate.restype = ctypes.c_int64
    lib.dcg_server_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int32, ctypes.c_int64,
                                      P(ctypes.c_void_p)]
    lib.dcg_server_submit.argtypes = [ctypes.c_void_p, P(_System), ctypes.c_uint64]
    lib.dcg_server_poll.argtypes = [ctypes.c_void_p, ctypes.c_int32, P(_RequestResult)]
    lib.dcg_server_pending.argtypes = [ctypes.c_void_p, P(ctypes.c_int32), P(ctypes.c_int32)]
    lib.dcg_server_clock.argtypes = [ctypes.c_void_p]
    lib.dcg_server_clock.restype = ctypes.c_double
    lib.dcg_server_device_bytes.argtypes = [ctypes.c_void_p]
    lib.dcg_server_device_bytes.restype = ctypes.c_int64
    lib.dcg_server_destroy.argtypes = [ctypes.c_void_p]
    lib.dcg_casci_energy_check.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.dcg_autotune_mode.argtypes = [ctypes.c_int32]
    lib.dcg_set_autotune_trials.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    lib.dcg_set_merge_reductions.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    lib.dcg_merged_reduction_stats.argtypes = [ctypes.c_int, ctypes.c_void_p]
    lib.dcg_autotune_entries.argtypes = [ctypes.c_void_p, ctypes.c_int32]
    lib.dcg_autotune_entries.restype = ctypes.c_int32
    lib.dcg_ivo.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p,
                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, P(ctypes.c_int32)]
    lib.dcg_read_mrconee.argtypes = [ctypes.c_char_p, P(_ActiveInput), P(P(_Mrconee))]
    lib.dcg_free_mrconee.argtypes = [P(_Mrconee)]
    lib.dcg_free_mrconee.restype = None
    lib.dcg_read_mdcint.argtypes = [ctypes.c_char_p, P(_Mrconee), P(_ActiveInput), ctypes.c_int32,
                                    P(P(_MdcintRaw))]
    lib.dcg_free_mdcint.argtypes = [P(_MdcintRaw)]
    lib.dcg_free_mdcint.restype = None
    lib.dcg_io_last_error.restype = ctypes.c_char_p
    _lib = lib
    return lib


EXPORTED_SYMBOLS = ["dcg_create", "dcg_destroy", "dcg_last_error", "dcg_set_system", "dcg_casci",
                    "dcg_caspt2", "dcg_caspt2_irreps", "dcg_casci_determinants", "dcg_get_eps", "dcg_stage_times", "dcg_kernel_launches", "dcg_version",
                    "dcg_stream", "dcg_set_wait_limit", "dcg_time_family", "dcg_family_stats", "dcg_solve_h",
                    "dcg_solve_h_noalloc", "dcg_heev", "dcg_heev_range", "dcg_heev_batch", "dcg_stedc", "dcg_zgemm",
                    "dcg_mdcint_canonicalize", "dcg_mdcint_records", "dcg_set_system_mdcint",
                    "dcg_set_casci_solver", "dcg_casci_iterations", "dcg_set_metric_solver",
                    "dcg_gram_cholesky_blocks", "dcg_gram_deflated_blocks", "dcg_device_bytes", "dcg_trim", "dcg_footprint_estimate", "dcg_server_create",
                    "dcg_server_submit", "dcg_server_poll", "dcg_server_pending", "dcg_server_clock",
                    "dcg_server_device_bytes", "dcg_server_destroy", "dcg_read_mrconee", "dcg_free_mrconee",
                    "dcg_read_mdcint", "dcg_free_mdcint", "dcg_io_last_error", "dcg_ivo",
                    "dcg_autotune_mode", "dcg_autotune_entries", "dcg_set_autotune_trials",
                    "dcg_set_merge_reductions", "dcg_merged_reduction_stats",
                    "dcg_casci_energy_check"]
FAMILIES = {"none": 0, "transform": 1, "hstream": 2, "rdm": 3, "scatter": 4, "eig": 5, "eig_tri": 6,
            "eig_val": 7, "eig_vec": 8, "eig_back": 9, "split_mma": 10}


TUNE_KINDS = {1: "fp64_gemm_tile_ksplit", 2: "split_gemm_kernel_raster"}


def autotune_mode(mode: int = -1) -> int:
    """dcg_autotune_mode: 1 tune on first use, 0 heuristics, 2 clear the table; -1 query.
    Returns the previous mode."""
    return int(load_library().dcg_autotune_mode(int(mode)))


def autotune_entries() -> List[dict]:
    """The process-wide table of tuned choices (dcg_autotune_entries)."""
    lib = load_library()
    n = int(lib.dcg_autotune_entries(None, 0))
    buf = (_TuneEntry * max(n, 1))()
    n = int(lib.dcg_autotune_entries(ctypes.cast(buf, ctypes.c_void_p), n))
    return [dict(kind=TUNE_KINDS.get(e.kind, e.kind), ops=e.ops, m=e.m, n=e.n, k=e.k, flags=e.flags,
                 choice=e.choice, ncand=e.ncand, best_ms=round(e.best_ms, 4), heuristic_ms=round(e.heuristic_ms, 4))
            for e in buf[:n]]


def _ptr(a: Optional[np.ndarray], ct):
    if a is None:
        return ctypes.POINTER(ct)()
    return a.ctypes.data_as(ctypes.POINTER(ct))


@dataclasses.dataclass
class SystemInput:
    """What one solve consumes (the reference's module globals after its readers)."""
    ninact: int
    nact: int
    nsec: int
    nelec: int
    nmo: int
    nsymrpa: int
    multb: np.ndarray          # (2n, 2n) Fortran MULTB(i0,j0) at [i0-1, j0-1]
    irpamo: np.ndarray         # (nmo,) 1-based, CAS order
    h: np.ndarray              # (nmo, nmo) complex, CAS order
    ecore: float
    rec_idx: np.ndarray        # (n, 4) 1-based MDCINTNEW indices
    rec_val: np.ndarray        # (n,) complex (or float)
    realonly: bool
    totsym: int = 1
    selectroot: int = 1
    eshift: float = 0.0
    ras: Tuple[int, int, int] = (0, 0, 0)
    ras1_max_hole: int = 0
    ras3_max_elec: int = 0
    min_hole_ras1: int = 0
    min_elec_ras3: int = 0

    @classmethod
    def from_synth(cls, s, totsym: int = 1, selectroot: int = 1) -> "SystemInput":
        c = s.cfg
        return cls(ninact=c.ninact, nact=c.nact, nsec=c.nsec, nelec=c.nelec, nmo=s.nmo, nsymrpa=1,
                   multb=s.multb, irpamo=s.irpamo, h=s.h, ecore=s.ecore, rec_idx=s.rec_idx, rec_val=s.rec_val,
                   realonly=c.realonly, totsym=totsym, selectroot=selectroot, eshift=c.eshift)

    @classmethod
    def from_files(cls, directory: str, ciroot_index: int = 0) -> "SystemInput":
        from . import dirac_io
        inp = dirac_io.read_active_inp(os.path.join(directory, "active.inp"))
        mrc = dirac_io.read_mrconee(os.path.join(directory, "MRCONEE"), inp)
        new = dirac_io.read_mdcint_new(directory, mrc, inp)
        ts, sr = inp.ciroots[ciroot_index]
        return cls(ninact=inp.ninact, nact=inp.nact, nsec=inp.nsec, nelec=inp.nelec, nmo=mrc.nmo,
                   nsymrpa=mrc.nsymrpa, multb=mrc.multb, irpamo=mrc.irpamo, h=mrc.h, ecore=mrc.ecore,
                   rec_idx=new.idx, rec_val=new.val, realonly=new.realonly, totsym=ts, selectroot=sr,
                   eshift=inp.eshift, ras=(len(inp.ras1), len(inp.ras2), len(inp.ras3)),
                   ras1_max_hole=inp.ras1_max_hole, ras3_max_elec=inp.ras3_max_elec,
                   min_hole_ras1=inp.min_hole_ras1, min_elec_ras3=inp.min_elec_ras3)

    @classmethod
    def from_npz(cls, path: str) -> "SystemInput":
        z = np.load(path, allow_pickle=False)
        val = z["rec_re"] + 1j * z["rec_im"] if "rec_im" in z.files else z["rec_re"].astype(np.complex128)
        d = {k: z[k] for k in z.files}
        return cls(ninact=int(d["ninact"]), nact=int(d["nact"]), nsec=int(d["nsec"]), nelec=int(d["nelec"]),
                   nmo=int(d["nmo"]), nsymrpa=int(d["nsymrpa"]), multb=d["multb"], irpamo=d["irpamo"],
                   h=d["h_re"] + 1j * d["h_im"], ecore=float(d["ecore"]), rec_idx=d["rec_idx"].astype(np.int32),
                   rec_val=val, realonly=bool(d["realonly"]), totsym=int(d["totsym"]),
                   selectroot=int(d["selectroot"]), eshift=float(d["eshift"]),
                   ras=tuple(int(x) for x in d["ras"]), ras1_max_hole=int(d["ras1_max_hole"]),
                   ras3_max_elec=int(d["ras3_max_elec"]), min_hole_ras1=int(d["min_hole_ras1"]),
                   min_elec_ras3=int(d["min_elec_ras3"]))


class HostBuffers:
    """Arrays in the exact layout of ``dcg_system`` (kept alive for the call).

    ``pinned=True`` places the record arrays in page-locked memory (cudaHostAlloc through
    the CUDA runtime of the library's process) so the host-to-device copies run at link
    speed."""

    def __init__(self, s: SystemInput):
        self.multb = np.ascontiguousarray(np.asarray(s.multb).T, dtype=np.int32)   # column-major
        self.irpamo = np.ascontiguousarray(s.irpamo, dtype=np.int32)
        h = np.asarray(s.h, dtype=np.complex128)
        self.h_re = np.ascontiguousarray(h.real.T)
        self.h_im = np.ascontiguousarray(h.imag.T)
        self.ijkl = np.ascontiguousarray(s.rec_idx, dtype=np.int32)
        v = np.asarray(s.rec_val)
        self.re = np.ascontiguousarray(v.real, dtype=np.float64)
        self.im = None if s.realonly else np.ascontiguousarray(np.imag(v), dtype=np.float64)
        st = _System()
        st.ninact, st.nact, st.nsec, st.nelec = s.ninact, s.nact, s.nsec, s.nelec
        st.nmo, st.nsymrpa, st.totsym, st.selectroot = s.nmo, s.nsymrpa, s.totsym, s.selectroot
        st.realonly = int(bool(s.realonly))
        st.eshift, st.ecore = float(s.eshift), float(s.ecore)
        st.multb = _ptr(self.multb, ctypes.c_int32)
        st.irpamo = _ptr(self.irpamo, ctypes.c_int32)
        st.h_re = _ptr(self.h_re, ctypes.c_double)
        st.h_im = _ptr(self.h_im, ctypes.c_double)
        st.nrec = len(self.re)
        st.rec_ijkl = _ptr(self.ijkl, ctypes.c_int32)
        st.rec_re = _ptr(self.re, ctypes.c_double)
        st.rec_im = _ptr(self.im, ctypes.c_double)
        st.ras1_size, st.ras2_size, st.ras3_size = (int(x) for x in s.ras)
        st.ras1_max_hole, st.ras3_max_elec = s.ras1_max_hole, s.ras3_max_elec
        st.min_hole_ras1, st.min_elec_ras3 = s.min_hole_ras1, s.min_elec_ras3
        self.struct = st

    def rebind(self) -> None:
        """Re-point the struct at the current record arrays (e.g. after swapping them for
        page-locked copies)."""
        st = self.struct
        st.rec_ijkl = _ptr(self.ijkl, ctypes.c_int32)
        st.rec_re = _ptr(self.re, ctypes.c_double)
        st.rec_im = _ptr(self.im, ctypes.c_double)
        st.rec_on_device = 0

    def use_device_records(self, ijkl_ptr: int, re_ptr: int, im_ptr: int) -> None:
        """Point the record arrays at device memory already holding them (HBM-resident input)."""
        st = self.struct
        st.rec_ijkl = ctypes.cast(ctypes.c_void_p(ijkl_ptr), ctypes.POINTER(ctypes.c_int32))
        st.rec_re = ctypes.cast(ctypes.c_void_p(re_ptr), ctypes.POINTER(ctypes.c_double))
        st.rec_im = ctypes.cast(ctypes.c_void_p(im_ptr), ctypes.POINTER(ctypes.c_double)) if im_ptr else \
            ctypes.POINTER(ctypes.c_double)()
        st.rec_on_device = 1

    @property
    def record_bytes(self) -> int:
        return int(self.ijkl.nbytes + self.re.nbytes + (self.im.nbytes if self.im is not None else 0))

    @property
    def h2d_bytes(self) -> int:
        n = self.ijkl.nbytes + self.re.nbytes + (self.im.nbytes if self.im is not None else 0)
        return int(n + self.h_re.nbytes + self.h_im.nbytes + self.multb.nbytes + self.irpamo.nbytes)


@dataclasses.dataclass
class Caspt2Result:
    casci_energies: np.ndarray
    ndet: int
    e2: Dict[str, float]
    sumc2: Dict[str, float]
    e0: float
    total_energy: float
    stage_ms: Dict[str, float]
    kernel_launches: int
    # e2X(isym) of the symmetry blocks solve_X_subspace prints (subspaces A..G), by isym
    e2_sym: Dict[str, Dict[int, float]] = dataclasses.field(default_factory=dict)

    @property
    def e2_total(self) -> float:
        return float(sum(self.e2.values()))

    @property
    def sumc2_total(self) -> float:
        return float(sum(self.sumc2.values()))


class NativeFiles:
    """MRCONEE and MDCINT of a DIRAC run directory read by the library's C++ readers
    (dcg_read_mrconee / dcg_read_mdcint), without the Fortran driver or numpy parsing.

    ``inp`` is a dirac_io.ActiveInput; ``pinned`` puts the MDCINT entry arrays in page-locked
    memory.  ``mdcint`` can be passed to Caspt2Session.set_system_mdcint as is."""

    def __init__(self, directory: str, inp, pinned: bool = False, mdcint: bool = True):
        self.lib = load_library()
        self._ras = [np.ascontiguousarray(x, np.int32) for x in (inp.ras1, inp.ras2, inp.ras3)]
        a = _ActiveInput()
        a.ninact, a.nact, a.nsec, a.nelec = inp.ninact, inp.nact, inp.nsec, inp.nelec
        a.diracver = inp.diracver
        a.scheme = int(inp.scheme or 0)
        a.nras1, a.nras2, a.nras3 = (len(x) for x in self._ras)
        a.ras1, a.ras2, a.ras3 = (x.ctypes.data if len(x) else None for x in self._ras)
        self._inp = a
        self.inp = inp
        self._m = ctypes.POINTER(_Mrconee)()
        self._r = ctypes.POINTER(_MdcintRaw)()
        rc = self.lib.dcg_read_mrconee(os.path.join(directory, "MRCONEE").encode(), ctypes.byref(a),
                                       ctypes.byref(self._m))
        if rc != 0:
            raise DcgError(rc, self.lib.dcg_io_last_error().decode())
        self.realonly = None
        if not mdcint:
            return
        rc = self.lib.dcg_read_mdcint(directory.encode(), self._m, ctypes.byref(a), int(bool(pinned)),
                                      ctypes.byref(self._r))
        if rc != 0:
            self.close()
            raise DcgError(rc, self.lib.dcg_io_last_error().decode())
        self.realonly = bool(self._r.contents.realonly)

    @property
    def mdcint(self):
        """The dcg_mdcint_raw the reader filled (its storage lives as long as this object)."""
        return self._r.contents

    def mrconee(self):
        """The MRCONEE content as a dirac_io.MrconeeData (numpy copies)."""
        from .dirac_io import MrconeeData
        m = self._m.contents
        n, n2 = m.nmo, 2 * m.nsymrpa
        arr = lambda p, k: np.ctypeslib.as_array(p, shape=(k,)).copy()
        h = arr(m.h_re, n * n).reshape(n, n).T + 1j * arr(m.h_im, n * n).reshape(n, n).T
        return MrconeeData(nmo=n, ecore=m.ecore, nsymrpa=m.nsymrpa, repna=[],
                           multb=arr(m.multb, n2 * n2).reshape(n2, n2).T.astype(np.int64),
                           irpamo=arr(m.irpamo, n).astype(np.int64), mo_energy=arr(m.mo_energy, n),
                           dirac_to_cas=arr(m.dirac_to_cas, n + 1).astype(np.int64),
                           cas_to_dirac=arr(m.cas_to_dirac, n + 1).astype(np.int64), h=h,
                           hf_energy=m.hf_energy, dirac_32bit=bool(m.dirac_32bit))

    def raw(self):
        """The MDCINT records as a dirac_io.MdcintRaw (numpy copies)."""
        from .dirac_io import MdcintRaw
        r = self._r.contents
        def arr(addr, ct, k):
            if k == 0:
                return np.zeros(0, np.dtype(ct))
            return np.ctypeslib.as_array(ctypes.cast(addr, ctypes.POINTER(ct)), shape=(k,)).copy()
        ne = int(r.nent)
        return MdcintRaw(rec_ikr=arr(r.ikr, ctypes.c_int32, r.nrec), rec_jkr=arr(r.jkr, ctypes.c_int32, r.nrec),
                         rec_off=arr(r.rec_off, ctypes.c_int64, r.nrec + 1), indk=arr(r.indk, ctypes.c_int32, ne),
                         indl=arr(r.indl, ctypes.c_int32, ne), re=arr(r.re, ctypes.c_double, ne),
                         im=arr(r.im, ctypes.c_double, ne) if r.im else np.zeros(ne),
                         kr=arr(r.kr, ctypes.c_int32, 2 * r.nkr).reshape(r.nkr, 2), nmo=int(r.nmo),
                         dirac_to_cas=arr(r.dirac_to_cas, ctypes.c_int32, r.nmo + 1), scheme=int(r.scheme),
                         realonly=bool(r.realonly))

    def system_input(self, ciroot_index: int = 0) -> "SystemInput":
        """The SystemInput of this run directory without records (pass ``mdcint`` to
        Caspt2Session.set_system_mdcint, which builds them on the device)."""
        inp = self.inp
        m = self.mrconee()
        ts, sr = inp.ciroots[ciroot_index] if inp.ciroots else (1, 1)
        return SystemInput(ninact=inp.ninact, nact=inp.nact, nsec=inp.nsec, nelec=inp.nelec, nmo=m.nmo,
                           nsymrpa=m.nsymrpa, multb=m.multb, irpamo=m.irpamo, h=m.h, ecore=m.ecore,
                           rec_idx=np.zeros((0, 4), np.int32), rec_val=np.zeros(0, np.complex128),
                           realonly=self.realonly, totsym=ts, selectroot=sr, eshift=inp.eshift,
                           ras=(len(inp.ras1), len(inp.ras2), len(inp.ras3)), ras1_max_hole=inp.ras1_max_hole,
                           ras3_max_elec=inp.ras3_max_elec, min_hole_ras1=inp.min_hole_ras1,
                           min_elec_ras3=inp.min_elec_ras3)

    def close(self) -> None:
        if getattr(self, "_r", None):
            self.lib.dcg_free_mdcint(self._r)
            self._r = ctypes.POINTER(_MdcintRaw)()
        if getattr(self, "_m", None):
            self.lib.dcg_free_mrconee(self._m)
            self._m = ctypes.POINTER(_Mrconee)()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Caspt2Session:
    def __init__(self, device: int = 0, precision: int = DCG_PREC_FP64):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.dcg_create(device, precision, ctypes.byref(h))
        if rc != 0:
            raise DcgError(rc, "dcg_create failed (no usable CUDA device?)")
        self.h = h
        self._bufs: Optional[HostBuffers] = None
        self.system: Optional[SystemInput] = None

    def close(self):
        if self.h:
            self.lib.dcg_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != 0:
            msg = self.lib.dcg_last_error(self.h)
            raise DcgError(rc, msg.decode() if msg else "")

    def set_system(self, s: SystemInput, bufs: Optional[HostBuffers] = None) -> None:
        self._bufs = bufs or HostBuffers(s)
        self.system = s
        self._check(self.lib.dcg_set_system(self.h, ctypes.byref(self._bufs.struct)))

    def casci(self, nroot: int = 1, want_ci: bool = False):
        n = max(1, int(nroot))
        eig = np.zeros(n)
        nd = ctypes.c_int32(0)
        self._check(self.lib.dcg_casci(self.h, n, eig.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), None, None,
                                       ctypes.byref(nd)))
        ndet = nd.value
        eig = eig[:min(n, ndet)]
        if want_ci:
            nr = min(n, ndet)
            cr = np.zeros(ndet * nr)
            ci = np.zeros(ndet * nr)
            self._check(self.lib.dcg_casci(self.h, n, eig.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                           cr.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                           ci.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(nd)))
            return eig, ndet, (cr + 1j * ci).reshape(nr, ndet).T
        return eig, ndet

    def caspt2(self, skip_mask: int = 0) -> Tuple[Dict[str, float], Dict[str, float], float, float]:
        e2 = np.zeros(8)
        sc = np.zeros(8)
        e0 = ctypes.c_double(0.0)
        et = ctypes.c_double(0.0)
        dp = ctypes.POINTER(ctypes.c_double)
        self._check(self.lib.dcg_caspt2(self.h, ctypes.c_uint32(skip_mask), e2.ctypes.data_as(dp),
                                        sc.ctypes.data_as(dp), ctypes.byref(e0), ctypes.byref(et)))
        return ({k: float(e2[i]) for i, k in enumerate(SUBSPACES)},
                {k: float(sc[i]) for i, k in enumerate(SUBSPACES)}, e0.value, et.value)

    def caspt2_irreps(self) -> Tuple[Dict[str, Dict[int, float]], np.ndarray, np.ndarray, np.ndarray]:
        """Per-irrep results of the last caspt2 (dcg_caspt2_irreps): the printed e2X(isym)
        values as {subspace: {isym: e2}}, and the raw (8, nsym) arrays e2, sumc2, printed."""
        ns = int(self.system.nsymrpa)
        e2 = np.zeros((8, ns))
        sc = np.zeros((8, ns))
        pr = np.zeros((8, ns), np.int32)
        self._check(self.lib.dcg_caspt2_irreps(self.h, ns, e2.ctypes.data, sc.ctypes.data, pr.ctypes.data))
        out = {k: {q + 1: float(e2[i, q]) for q in range(ns) if pr[i, q]} for i, k in enumerate(SUBSPACES)}
        return {k: v for k, v in out.items() if v}, e2, sc, pr

    def casci_determinants(self, ndet: int) -> np.ndarray:
        """Bit strings of the CASCI determinants in the reference's dict order."""
        out = np.zeros(max(1, ndet), np.int64)
        self._check(self.lib.dcg_casci_determinants(self.h, out.ctypes.data, len(out)))
        return out[:ndet]

    def eps(self) -> np.ndarray:
        n = self.system.nmo
        out = np.zeros(n)
        self._check(self.lib.dcg_get_eps(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), n))
        return out

    def stage_ms(self) -> Dict[str, float]:
        out = np.zeros(len(STAGES))
        k = self.lib.dcg_stage_times(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(STAGES))
        return {STAGES[i]: float(out[i]) for i in range(k)}

    def kernel_launches(self) -> int:
        return int(self.lib.dcg_kernel_launches(self.h))

    def mdcint_canonicalize(self, raw):
        """MDCINT records -> the MDCINTNEW stream on the device (dcg_mdcint_canonicalize),
        copied back as a dirac_io.MdcintNew."""
        from .dirac_io import MdcintNew
        mb = raw if isinstance(raw, MdcintBuffers) else MdcintBuffers(raw)
        n = ctypes.c_int64(0)
        self._check(self.lib.dcg_mdcint_canonicalize(self.h, ctypes.byref(mb.struct), ctypes.byref(n)))
        idx = np.zeros((n.value, 4), np.int32)
        re = np.zeros(n.value)
        im = np.zeros(n.value)
        self._check(self.lib.dcg_mdcint_records(self.h, idx.ctypes.data, re.ctypes.data, im.ctypes.data))
        return MdcintNew(idx=idx, val=re + 1j * im, realonly=mb.realonly)

    def set_system_mdcint(self, s: SystemInput, raw) -> None:
        """dcg_set_system_mdcint: the system with its records built on the device from MDCINT
        (a dirac_io.MdcintRaw, MdcintBuffers, or the NativeFiles reader's ``mdcint``)."""
        if isinstance(raw, NativeFiles):
            raw = raw.mdcint
        if isinstance(raw, _MdcintRaw):
            mb, st = raw, raw
        else:
            mb = raw if isinstance(raw, MdcintBuffers) else MdcintBuffers(raw)
            st = mb.struct
        self._bufs = HostBuffers(s)
        self.system = s
        self._mdcint = mb
        self._check(self.lib.dcg_set_system_mdcint(self.h, ctypes.byref(self._bufs.struct), ctypes.byref(st)))

    def casci_energy_check(self) -> Dict[str, float]:
        """dcg_casci_energy_check: the e0test terms of the selected root after casci()."""
        out = np.zeros(8)
        self._check(self.lib.dcg_casci_energy_check(self.h, out.ctypes.data))
        keys = ("energyHF1", "energyHF2", "energy1", "energy2", "energy3", "energy4", "t_energy", "error")
        return {k: float(v) for k, v in zip(keys, out)}

    def ivo(self, nfsym: int, mo_energy: np.ndarray, nhomo: int = 0):
        """dcg_ivo: (eps (nsec,), U (nsec, nsec) complex, block_isym (nsec,), numh) of the
        improved virtual orbitals of the resident system."""
        ns = self.system.nsec
        me = np.ascontiguousarray(mo_energy, np.float64)
        eps = np.zeros(ns)
        ure = np.zeros((ns, ns), order="F")
        uim = np.zeros((ns, ns), order="F")
        bs = np.zeros(ns, np.int32)
        numh = ctypes.c_int32(0)
        self._check(self.lib.dcg_ivo(self.h, int(nfsym), me.ctypes.data, int(nhomo), eps.ctypes.data, ure.ctypes.data,
                                     uim.ctypes.data, bs.ctypes.data, ctypes.byref(numh)))
        return eps, ure + 1j * uim, bs, numh.value

    def set_casci_solver(self, solver: str) -> None:
        """CASCI eigensolver: "auto", "dense" or "davidson" (dcg_set_casci_solver)."""
        self._check(self.lib.dcg_set_casci_solver(self.h, CASCI_SOLVERS[solver]))

    def set_metric_solver(self, solver: str) -> None:
        """Gram-route metric of A and C: "auto" (Cholesky when no eigenvalue falls under the
        cutoff) or "eigen" (dcg_set_metric_solver)."""
        self._check(self.lib.dcg_set_metric_solver(self.h, METRIC_SOLVERS[solver]))

    def gram_cholesky_blocks(self) -> int:
        """Gram blocks of the last caspt2 solved by the Cholesky route."""
        return int(self.lib.dcg_gram_cholesky_blocks(self.h))

    def gram_deflated_blocks(self) -> int:
        """Gram blocks of the last caspt2 solved on the complement of deflated eigenvectors."""
        return int(self.lib.dcg_gram_deflated_blocks(self.h))

    def casci_iterations(self) -> int:
        """Davidson iterations of the last casci (0: dense solver)."""
        return int(self.lib.dcg_casci_iterations(self.h))

    def device_bytes(self) -> int:
        """Device bytes the context holds (dcg_device_bytes)."""
        return int(self.lib.dcg_device_bytes(self.h))

    def trim(self) -> None:
        """Release the context's device workspace (dcg_trim)."""
        self._check(self.lib.dcg_trim(self.h))

    def heev(self, a: np.ndarray, vectors: bool = True):
        """Hermitian eigendecomposition on the device (dcg_heev): ascending eigenvalues and,
        when ``vectors``, the eigenvectors as columns.  Reads the upper triangle of ``a``."""
        a = np.asarray(a)
        n = a.shape[0]
        are = np.asfortranarray(a.real, dtype=np.float64)
        aim = np.asfortranarray(a.imag, dtype=np.float64) if np.iscomplexobj(a) else None
        w = np.zeros(n)
        zr = np.zeros((n, n), order="F") if vectors else None
        zi = np.zeros((n, n), order="F") if vectors else None
        ptr = lambda x: None if x is None else x.ctypes.data
        self._check(self.lib.dcg_heev(self.h, n, ptr(are), ptr(aim), ptr(w), ptr(zr), ptr(zi)))
        return (w, zr + 1j * zi) if vectors else w

    def zgemm(self, precision: int, M: int, N: int, K: int, batch: int, A_ptr: int, a_si: int, a_sk: int, a_sb: int,
              B_ptr: int, ldb: int, conj_b: bool, C_ptr: int, c_si: int, c_sj: int, c_sb: int,
              accumulate: bool = False):
        """Complex GEMM on device buffers (dcg_zgemm); strides in complex elements."""
        self._check(self.lib.dcg_zgemm(self.h, precision, M, N, K, batch, A_ptr, a_si, a_sk, a_sb, B_ptr, ldb,
                                       int(conj_b), C_ptr, c_si, c_sj, c_sb, int(accumulate)))

    def heev_batch(self, mats):
        """Batched Hermitian eigendecompositions (dcg_heev_batch): list of (w, Z)."""
        k = len(mats)
        n = (ctypes.c_int32 * k)(*[m.shape[0] for m in mats])
        keep = []
        def arr(x):
            keep.append(x)
            return x.ctypes.data
        re = (ctypes.c_void_p * k)(*[arr(np.asfortranarray(m.real, dtype=np.float64)) for m in mats])
        im = (ctypes.c_void_p * k)(*[arr(np.asfortranarray(m.imag, dtype=np.float64)) for m in mats])
        ws = [np.zeros(m.shape[0]) for m in mats]
        zr = [np.zeros(m.shape, order="F") for m in mats]
        zi = [np.zeros(m.shape, order="F") for m in mats]
        wp = (ctypes.c_void_p * k)(*[w.ctypes.data for w in ws])
        zrp = (ctypes.c_void_p * k)(*[z.ctypes.data for z in zr])
        zip_ = (ctypes.c_void_p * k)(*[z.ctypes.data for z in zi])
        self._check(self.lib.dcg_heev_batch(self.h, k, n, re, im, wp, zrp, zip_))
        return [(w, a + 1j * b) for w, a, b in zip(ws, zr, zi)]

    def heev_range(self, a: np.ndarray, vlo: int):
        """Eigenvalues (all) and the eigenvectors of eigenvalues vlo..n-1 (dcg_heev_range)."""
        a = np.asarray(a)
        n = a.shape[0]
        are = np.asfortranarray(a.real, dtype=np.float64)
        aim = np.asfortranarray(a.imag, dtype=np.float64) if np.iscomplexobj(a) else None
        w = np.zeros(n)
        zr = np.zeros((n, n - vlo), order="F")
        zi = np.zeros((n, n - vlo), order="F")
        self._check(self.lib.dcg_heev_range(self.h, n, are.ctypes.data, None if aim is None else aim.ctypes.data,
                                            w.ctypes.data, vlo, zr.ctypes.data, zi.ctypes.data))
        return w, zr + 1j * zi

    def stedc(self, d: np.ndarray, e: np.ndarray, vectors: bool = True):
        """Symmetric tridiagonal eigendecomposition on the device (dcg_stedc)."""
        d = np.ascontiguousarray(d, dtype=np.float64)
        e = np.ascontiguousarray(e, dtype=np.float64)
        n = d.shape[0]
        w = np.zeros(n)
        z = np.zeros((n, n), order="F") if vectors else None
        self._check(self.lib.dcg_stedc(self.h, n, d.ctypes.data, e.ctypes.data if n > 1 else None, w.ctypes.data,
                                       z.ctypes.data if vectors else None))
        return (w, z) if vectors else w

    def solve_h(self, hclass_ptr: int, ninact: int, nsec: int, eps_i_ptr: int, eps_s_ptr: int, irp_i_ptr: int,
                irp_s_ptr: int, md_ptr: int, ms_ptr: int, nsymrpa: int, eshift: float) -> Tuple[float, float]:
        """solve_H_subspace on device-resident inputs (all *_ptr are device addresses)."""
        out = np.zeros(2)
        self._check(self.lib.dcg_solve_h(self.h, hclass_ptr, ninact, nsec, eps_i_ptr, eps_s_ptr, irp_i_ptr,
                                         irp_s_ptr, md_ptr, ms_ptr, nsymrpa, eshift,
                                         out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return float(out[0]), float(out[1])

    @property
    def stream_ptr(self) -> int:
        return int(self.lib.dcg_stream(self.h) or 0)

    def set_wait_limit(self, seconds: float) -> None:
        """dcg_set_wait_limit: time limit of the device-side waits that can give up (0: defaults)."""
        self._check(self.lib.dcg_set_wait_limit(self.h, float(seconds)))

    def time_family(self, family: str) -> None:
        self._check(self.lib.dcg_time_family(self.h, FAMILIES[family]))

    def family_stats(self) -> Tuple[float, int, float]:
        ms = ctypes.c_double(0.0)
        n = ctypes.c_int64(0)
        w = ctypes.c_double(0.0)
        self._check(self.lib.dcg_family_stats(self.h, ctypes.byref(ms), ctypes.byref(n), ctypes.byref(w)))
        return ms.value, n.value, w.value

    def solve(self, s: SystemInput, nroot: int = 1, skip_mask: int = 0,
              bufs: Optional[HostBuffers] = None) -> Caspt2Result:
        """set_system + casci + caspt2 for one (totsym, selectroot) entry."""
        self.set_system(s, bufs)
        eig, ndet = self.casci(max(nroot, s.selectroot))
        e2, sc2, e0, et = self.caspt2(skip_mask)
        return Caspt2Result(casci_energies=eig, ndet=ndet, e2=e2, sumc2=sc2, e0=e0, total_energy=et,
                            stage_ms=self.stage_ms(), kernel_launches=self.kernel_launches(),
                            e2_sym=self.caspt2_irreps()[0])


def merged_reduction_stats(device: int = 0) -> Dict[str, int]:
    """dcg_merged_reduction_stats: joint cooperative launches of the serving slots' reductions."""
    out = np.zeros(3, np.int64)
    rc = load_library().dcg_merged_reduction_stats(device, out.ctypes.data)
    if rc != 0:
        raise DcgError(rc, "dcg_merged_reduction_stats")
    return {"launches": int(out[0]), "joint_launches": int(out[1]), "submissions": int(out[2])}


def footprint_estimate(bufs: "HostBuffers") -> int:
    """dcg_footprint_estimate: upper estimate of one solve's device bytes in a fresh context."""
    return int(load_library().dcg_footprint_estimate(ctypes.byref(bufs.struct)))


@dataclasses.dataclass
class ServedResult:
    """One finished request of a ``Caspt2Server`` (times in seconds on the server clock)."""
    request_id: int
    status: int
    ndet: int
    casci_energy: float
    e2: Dict[str, float]
    sumc2: Dict[str, float]
    e0: float
    total_energy: float
    t_submit: float
    t_start: float
    t_end: float
    slot: int
    attempts: int
    error: str = ""

    @property
    def latency(self) -> float:
        return self.t_end - self.t_submit

    @property
    def e2_total(self) -> float:
        return float(sum(self.e2.values()))


class Caspt2Server:
    """The library's serving loop (dcg_server_*): ``slots`` contexts with a worker thread and a
    CUDA stream each, admission of queued requests by an HBM budget, results polled as they
    finish.  A request is one (system, selectroot) entry run as set_system + casci + caspt2.

    ``submit`` keeps the request's HostBuffers (and, through them, any device records) alive
    until its result has been polled."""

    def __init__(self, device: int = 0, precision: int = DCG_PREC_FP64, slots: int = 4, hbm_budget: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        rc = self.lib.dcg_server_create(device, precision, slots, int(hbm_budget), ctypes.byref(h))
        if rc != 0:
            raise DcgError(rc, "dcg_server_create failed")
        self.h = h
        self.slots = slots
        self._inflight: Dict[int, HostBuffers] = {}

    def submit(self, request_id: int, system, selectroot: Optional[int] = None) -> None:
        bufs = system if isinstance(system, HostBuffers) else HostBuffers(system)
        if selectroot is not None:
            bufs.struct.selectroot = int(selectroot)
        self._inflight[int(request_id)] = bufs
        rc = self.lib.dcg_server_submit(self.h, ctypes.byref(bufs.struct), ctypes.c_uint64(int(request_id)))
        if rc != 0:
            del self._inflight[int(request_id)]
            raise DcgError(rc, "request does not fit the server's device-memory budget" if rc == -5 else
                           "dcg_server_submit failed")

    def poll(self, timeout_ms: int = 0) -> Optional[ServedResult]:
        r = _RequestResult()
        rc = self.lib.dcg_server_poll(self.h, int(timeout_ms), ctypes.byref(r))
        if rc == 1:
            return None
        if rc != 0:
            raise DcgError(rc, "dcg_server_poll failed")
        self._inflight.pop(int(r.request_id), None)
        return ServedResult(request_id=int(r.request_id), status=int(r.status), ndet=int(r.ndet),
                            casci_energy=float(r.casci_energy),
                            e2={k: float(r.e2[i]) for i, k in enumerate(SUBSPACES)},
                            sumc2={k: float(r.sumc2[i]) for i, k in enumerate(SUBSPACES)}, e0=float(r.e0),
                            total_energy=float(r.etotal), t_submit=float(r.t_submit), t_start=float(r.t_start),
                            t_end=float(r.t_end), slot=int(r.slot), attempts=int(r.attempts),
                            error=r.error.decode(errors="replace"))

    def pending(self) -> Tuple[int, int]:
        q = ctypes.c_int32(0)
        r = ctypes.c_int32(0)
        self.lib.dcg_server_pending(self.h, ctypes.byref(q), ctypes.byref(r))
        return q.value, r.value

    def clock(self) -> float:
        return float(self.lib.dcg_server_clock(self.h))

    def device_bytes(self) -> int:
        return int(self.lib.dcg_server_device_bytes(self.h))

    def close(self) -> None:
        if self.h:
            self.lib.dcg_server_destroy(self.h)
            self.h = None
            self._inflight.clear()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def format_reference_lines(r: Caspt2Result, s: SystemInput) -> List[str]:
    """The reference's printed energy lines (casci.F90:77, solve_X_subspace e2/sumc2 lines,
    r4dcaspt2_tra.F90:437-442)."""
    out = [f"CASCI Total Energy ROOT{k + 1}{e:30.20f} a.u." for k, e in enumerate(r.casci_energies)]
    for k in SUBSPACES:
        if k != "H" and k in r.e2:
            # solve_X_subspace: the header and one line per printed symmetry block
            # (solve_A_subspace.F90:89,262/908: the real variant of A has two spaces before '=')
            out.append(f" e2{k.lower()}(isym)")
            gap = "  " if k == "B" or (k == "A" and s.realonly) else " "
            for q, v in sorted(r.e2_sym.get(k, {}).items()):
                out.append(f" e2{k.lower()}({q:3d}){gap}= {_e25(v)} a.u.")
        if k in r.e2:
            out.append(f" e2{k.lower()}      = {_e25(r.e2[k])} a.u.")
            out.append(f" sumc2,{k.lower()}  = {_e25(r.sumc2[k])}")
    sumc2 = r.sumc2_total
    out.append(f" c^2 is                         {sumc2:30.20f}")
    out.append(f" weight of 0th wave function is {1.0 / (1.0 + sumc2):30.20f}")
    out.append(f" Total second order energy is   {r.e2_total - s.eshift * sumc2:30.20f} a.u.")
    out.append(f" Total energy is                {r.total_energy:30.20f} a.u.")
    return out


def _e25(x: float) -> str:
    """Fortran E25.15 (0.ddddE+xx form)."""
    if x == 0.0:
        return f"{'0.000000000000000E+00':>25}"
    m, e = f"{x:.14E}".split("E")
    ex = int(e) + 1
    sign = "-" if x < 0 else ""
    digits = m.replace("-", "").replace(".", "")
    return f"{sign + '0.' + digits[:15] + f'E{ex:+03d}':>25}"


def run_case(directory: str, device: int = 0, precision: int = DCG_PREC_FP64, verbose: bool = True):
    """The reference's CASCI+CASPT2 flow for every .caspt2_ciroots entry of a case directory."""
    from . import dirac_io
    inp = dirac_io.read_active_inp(os.path.join(directory, "active.inp"))
    results = []
    with Caspt2Session(device, precision) as ses:
        for k in range(len(inp.ciroots)):
            s = SystemInput.from_files(directory, k)
            ses.set_system(s)
            eig, ndet = ses.casci(s.selectroot)
            chk = ses.casci_energy_check()   # r4dcasci's e0test (r4dcasci.F90:89)
            e2, sc2, e0, et = ses.caspt2()
            r = Caspt2Result(casci_energies=eig, ndet=ndet, e2=e2, sumc2=sc2, e0=e0, total_energy=et,
                             stage_ms=ses.stage_ms(), kernel_launches=ses.kernel_launches(),
                             e2_sym=ses.caspt2_irreps()[0])
            if verbose:
                print("\n".join(format_e0test_lines(chk, s.selectroot)))
                print("\n".join(format_reference_lines(r, s)))
            results.append(r)
    return results


def format_e0test_lines(chk: Dict[str, float], selectroot: int) -> List[str]:
    """e0test's energy lines (e0test.F90:92-96, 262-268), real parts."""
    return [f" energyHF(1) {chk['energyHF1']:30.17f}", f" energyHF(2) {chk['energyHF2']:30.17f}",
            f"selectroot {selectroot}"] + [f" energy {q} = {chk[f'energy{q}']:30.17f}" for q in range(1, 5)] + \
           [f" t-energy(1-4) {chk['t_energy']:30.17f}", f" C the error {chk['error']:30.17e}"]
