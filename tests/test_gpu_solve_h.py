"""dcg_solve_h (solve_H_subspace on a caller's device-resident H class) against a numpy
evaluation of the same sum, with and without point-group symmetry."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _numpy_h(H, eps_i, eps_s, irp_i, irp_s, md, ms, eshift):
    ns, ni = len(eps_s), len(eps_i)
    e2 = sc = 0.0
    for a in range(ns):
        for b in range(a):
            for i in range(ni):
                for j in range(i):
                    if ms[md[irp_s[a] - 1, irp_i[i] - 1] - 1, md[irp_s[b] - 1, irp_i[j] - 1] - 1] != 1:
                        continue
                    v = H[a, i, b, j] - H[a, j, b, i]
                    e = eps_s[a] + eps_s[b] - eps_i[i] - eps_i[j] + eshift
                    e2 -= abs(v) ** 2 / e
                    sc += abs(v / e) ** 2
    return e2, sc


@pytest.mark.parametrize("nsym", [1, 2])
def test_solve_h_matches_numpy(gpu_lib, nsym):
    torch = pytest.importorskip("torch")
    from dirac_caspt2_gb300 import api
    rng = np.random.default_rng(7 + nsym)
    ni, ns = 6, 10
    H = (rng.normal(size=(ns, ni, ns, ni)) + 1j * rng.normal(size=(ns, ni, ns, ni))) * 0.01
    eps_i = np.sort(rng.uniform(-5, -1, ni))
    eps_s = np.sort(rng.uniform(0.5, 9, ns))
    irp_i = rng.integers(1, nsym + 1, ni).astype(np.int32)
    irp_s = rng.integers(1, nsym + 1, ns).astype(np.int32)
    if nsym == 1:
        md = np.ones((1, 1), np.int32)
        ms = np.ones((1, 1), np.int32)
    else:
        md = np.array([[2, 1], [1, 2]], np.int32)
        ms = np.array([[1, 2], [2, 1]], np.int32)
    ref = _numpy_h(H, eps_i, eps_s, irp_i, irp_s, md, ms, 0.05)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    Hd = dev(np.asfortranarray(H).ravel(order="F").view(np.float64))
    tensors = [Hd, dev(eps_i), dev(eps_s), dev(irp_i), dev(irp_s), dev(md), dev(ms)]
    with api.Caspt2Session(0) as ses:
        got = ses.solve_h(*[t.data_ptr() for t in tensors[:1]], ni, ns, *[t.data_ptr() for t in tensors[1:]],
                          nsym, 0.05)
    assert abs(got[0] - ref[0]) < 1e-13 * max(1.0, abs(ref[0]))
    assert abs(got[1] - ref[1]) < 1e-13 * max(1.0, abs(ref[1]))
