"""dcg_solve_h_noalloc: the H-subspace sum for callers that cannot allocate device memory
(their device memory comes from their own pool or another runtime's allocator), checked
through the C ABI against the allocating entry point dcg_solve_h on the same device data,
on two calls in a row (the static scratch keeps the previous call's contents), up to the
largest size the scratch holds (ninact = 128: all 8128 inactive pairs)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13


def _inputs(torch, nsym, ni, ns, seed):
    rng = np.random.default_rng(seed)
    H = (rng.normal(size=(ns, ni, ns, ni)) + 1j * rng.normal(size=(ns, ni, ns, ni))) * 0.01
    eps_i = np.sort(rng.uniform(-5, -1, ni))
    eps_s = np.sort(rng.uniform(0.5, 9, ns))
    irp_i = rng.integers(1, nsym + 1, ni).astype(np.int32)
    irp_s = rng.integers(1, nsym + 1, ns).astype(np.int32)
    md = np.ones((1, 1), np.int32) if nsym == 1 else np.array([[2, 1], [1, 2]], np.int32)
    ms = np.ones((1, 1), np.int32) if nsym == 1 else np.array([[1, 2], [2, 1]], np.int32)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return [dev(np.asfortranarray(H).ravel(order="F").view(np.float64)), dev(eps_i), dev(eps_s), dev(irp_i),
            dev(irp_s), dev(md), dev(ms)]


def _noalloc(lib, t, ni, ns, nsym, eshift, stream):
    out = (ctypes.c_double * 2)()
    f = lib.dcg_solve_h_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32] + [ctypes.c_void_p] * 6 + \
                 [ctypes.c_int32, ctypes.c_double, ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)]
    rc = f(t[0].data_ptr(), ni, ns, t[1].data_ptr(), t[2].data_ptr(), t[3].data_ptr(), t[4].data_ptr(),
           t[5].data_ptr(), t[6].data_ptr(), nsym, eshift, stream, out)
    return rc, (out[0], out[1])


@pytest.mark.parametrize("nsym,ni,ns", [(1, 6, 10), (2, 8, 12), (1, 20, 40), (2, 128, 4)])
def test_noalloc_matches_allocating_entry(gpu_lib, nsym, ni, ns):
    torch = pytest.importorskip("torch")
    from dirac_caspt2_gb300 import api
    t = _inputs(torch, nsym, ni, ns, seed=ni + ns)
    torch.cuda.synchronize()
    with api.Caspt2Session(0) as ses:
        ref = ses.solve_h(t[0].data_ptr(), ni, ns, t[1].data_ptr(), t[2].data_ptr(), t[3].data_ptr(),
                          t[4].data_ptr(), t[5].data_ptr(), t[6].data_ptr(), nsym, 0.02)
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        rc, got = _noalloc(gpu_lib, t, ni, ns, nsym, 0.02, stream)
        assert rc == 0
        assert abs(got[0] - ref[0]) <= TOL * max(1.0, abs(ref[0]))
        assert abs(got[1] - ref[1]) <= TOL * max(1.0, abs(ref[1]))


def test_noalloc_rejects_too_many_inactive(gpu_lib):
    torch = pytest.importorskip("torch")
    t = _inputs(torch, 1, 2, 2, seed=1)
    rc, _ = _noalloc(gpu_lib, t, 129, 2, 1, 0.0, 0)
    assert rc == -1     # DCG_E_ARG: beyond the static scratch (ninact <= 128)
