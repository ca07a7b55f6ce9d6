"""The serving loop (dcg_server_*) on the GPU: each request's result in a mix of concurrently
running requests of different sizes equals the result of the same request solved alone in a
fresh context (bit-identical; stated tolerance 1e-12 Eh), also when the Householder reductions
of concurrent requests ran merged in joint cooperative launches, the HBM budget bounds what runs at
once, oversize requests are refused, and the footprint estimate bounds a solve's device
memory.  The systems come from the device generator (records resident in HBM); one of them is
also checked against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_MIX = 1e-12

SIZES = [(4, 4, 20, 2), (6, 6, 40, 3), (8, 8, 60, 4), (4, 6, 30, 3), (8, 4, 50, 2), (6, 8, 24, 4),
         (10, 6, 64, 3), (4, 8, 40, 4)]


@pytest.fixture(scope="module")
def stream(gpu_lib):
    import torch
    from dirac_caspt2_gb300 import synth, synth_device as sd
    out = []
    for k, (ni, na, ns, ne) in enumerate(SIZES):
        cfg = synth.SynthConfig(ni, na, ns, ne, seed=100 + k)
        out.append(sd.make_system_device(cfg, "cuda"))
    torch.cuda.synchronize()
    return out


@pytest.fixture(scope="module", params=["fp64", "split"])
def alone(request, stream):
    from dirac_caspt2_gb300 import api
    prec = api.DCG_PREC_SPLIT if request.param == "split" else api.DCG_PREC_FP64
    res = []
    for s in stream:
        with api.Caspt2Session(0, prec) as ses:
            res.append(ses.solve(s.system_input(), bufs=s.buffers()))
    return prec, res


def _same(served, r):
    from dirac_caspt2_gb300 import api
    d = [abs(served.casci_energy - r.casci_energies[-1]), abs(served.total_energy - r.total_energy),
         abs(served.e0 - r.e0)]
    d += [abs(served.e2[k] - r.e2[k]) for k in api.SUBSPACES]
    d += [abs(served.sumc2[k] - r.sumc2[k]) for k in api.SUBSPACES]
    return max(d)


def test_mix_equals_alone(stream, alone):
    """All requests queued at once on 4 slots (several run concurrently, on separate streams)."""
    from dirac_caspt2_gb300 import api
    prec, ref = alone
    m0 = api.merged_reduction_stats(0)
    with api.Caspt2Server(0, prec, slots=4) as srv:
        for rep in range(2):   # the second pass reuses the slots' resident workspaces
            for k, s in enumerate(stream):
                srv.submit(rep * 100 + k, s.buffers())
            got = {}
            while len(got) < len(stream):
                r = srv.poll(60000)
                assert r is not None, "served request did not finish within 60 s"
                got[r.request_id] = r
            spans = sorted((r.t_start, r.t_end) for r in got.values())
            overlap = any(spans[i + 1][0] < spans[i][1] for i in range(len(spans) - 1))
            assert overlap, "no two requests ran at the same time"
            assert len({r.slot for r in got.values()}) > 1
            for k in range(len(stream)):
                r = got[rep * 100 + k]
                assert r.status == 0
                assert r.ndet == ref[k].ndet
                assert _same(r, ref[k]) <= TOL_MIX, (k, _same(r, ref[k]))
    # the slots' Householder reductions went through the batcher (whether two requests met in
    # one launch depends on timing; tests/test_gpu_merge.py makes them meet)
    m1 = api.merged_reduction_stats(0)
    assert m1["launches"] > m0["launches"]


def test_budget_serialises(stream, gpu_lib):
    """A budget that holds one request at a time (four copies of one request, budget 1.5 times
    its estimate): the requests run one after another."""
    from dirac_caspt2_gb300 import api
    bufs = [stream[2].buffers() for _ in range(4)]
    est = api.footprint_estimate(bufs[0])
    with api.Caspt2Server(0, api.DCG_PREC_FP64, slots=4, hbm_budget=int(1.5 * est)) as srv:
        for k, b in enumerate(bufs):
            srv.submit(k, b)
        got = []
        while len(got) < len(bufs):
            r = srv.poll(60000)
            assert r is not None
            got.append(r)
    assert all(r.status == 0 for r in got)
    spans = sorted((r.t_start, r.t_end) for r in got)
    assert all(spans[i + 1][0] >= spans[i][1] for i in range(len(spans) - 1)), spans


def test_oversize_refused(stream):
    from dirac_caspt2_gb300 import api
    with api.Caspt2Server(0, api.DCG_PREC_FP64, slots=1, hbm_budget=1 << 20) as srv:
        with pytest.raises(api.DcgError) as e:
            srv.submit(1, stream[0].buffers())
        assert e.value.code == -5
        assert srv.pending() == (0, 0)


def test_footprint_estimate_bounds(stream):
    """dcg_footprint_estimate is an upper bound of a fresh context's device bytes after a solve."""
    from dirac_caspt2_gb300 import api
    for prec in (api.DCG_PREC_FP64, api.DCG_PREC_SPLIT):
        for s in stream:
            b = s.buffers()
            with api.Caspt2Session(0, prec) as ses:
                ses.solve(s.system_input(), bufs=b)
                used = ses.device_bytes()
            est = api.footprint_estimate(b)
            assert 0 < used <= est, (s.cfg, used, est)


@pytest.mark.parametrize("dims", [(24, 4, 400, 2), (4, 12, 60, 6)])
def test_footprint_estimate_bounds_larger(gpu_lib, dims):
    """The same bound on a large secondary space (its split slices) and on 12 active spinors
    (their densities)."""
    import torch
    from dirac_caspt2_gb300 import api, synth, synth_device as sd
    s = sd.make_system_device(synth.SynthConfig(*dims, seed=3), "cuda")
    torch.cuda.synchronize()
    b = s.buffers()
    est = api.footprint_estimate(b)
    for prec in (api.DCG_PREC_FP64, api.DCG_PREC_SPLIT):
        with api.Caspt2Session(0, prec) as ses:
            ses.solve(s.system_input(), bufs=b)
            used = ses.device_bytes()
        assert 0 < used <= est, (dims, prec, used, est)


def test_trim_and_resolve(stream, alone):
    from dirac_caspt2_gb300 import api
    prec, ref = alone
    s = stream[2]
    with api.Caspt2Session(0, prec) as ses:
        r1 = ses.solve(s.system_input(), bufs=s.buffers())
        assert ses.device_bytes() > 0
        ses.trim()
        assert ses.device_bytes() == 0
        r2 = ses.solve(s.system_input(), bufs=s.buffers())
    assert r1.total_energy == r2.total_energy == ref[2].total_energy


def test_device_generated_system_vs_oracle(stream, gpu_lib):
    """A device-generated request solved through the server matches the oracle on the same
    integrals (records copied back to the host for the oracle)."""
    from dirac_caspt2_gb300 import api
    from oracle import caspt2_oracle as O
    from conftest import oracle_system
    s = stream[0]
    si = s.system_input()
    si.rec_idx = s.rec_idx.cpu().numpy()
    si.rec_val = s.rec_re.cpu().numpy() + 1j * s.rec_im.cpu().numpy()
    ref = O.run(oracle_system(si))
    with api.Caspt2Server(0, api.DCG_PREC_FP64, slots=2) as srv:
        srv.submit(7, s.buffers())
        r = srv.poll(60000)
    assert r is not None and r.status == 0
    assert abs(r.casci_energy - ref.casci_energies[si.selectroot - 1]) <= 1e-9
    for k in api.SUBSPACES:
        assert abs(r.e2[k] - ref.e2.get(k, 0.0)) <= 1e-9, k
    assert abs(r.total_energy - ref.total_energy) <= 1e-9
