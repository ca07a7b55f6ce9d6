"""The autotuner: a solve with tuning on fills the process-wide table (FP64 GEMM tiles and
K-splits, split GEMM rasters) and gives the energies of the heuristic choices within
summation-order rounding; a context with trials off adds no entries; mode 2 clears."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tuned_solve_matches_heuristic(gpu_lib):
    from dirac_caspt2_gb300 import api, synth
    s = api.SystemInput.from_synth(synth.make_system(synth.SynthConfig(16, 8, 240, 4, seed=21)))
    prev = api.autotune_mode(0)
    try:
        api.autotune_mode(2)
        with api.Caspt2Session(0, api.DCG_PREC_SPLIT) as ses:
            ref = ses.solve(s)
        assert api.autotune_entries() == []
        api.autotune_mode(1)
        with api.Caspt2Session(0, api.DCG_PREC_SPLIT) as ses:
            ses.lib.dcg_set_autotune_trials(ses.h, 0)
            r0 = ses.solve(s)
        assert api.autotune_entries() == []          # no trials in that context
        assert r0.total_energy == ref.total_energy
        with api.Caspt2Session(0, api.DCG_PREC_SPLIT) as ses:
            r1 = ses.solve(s)
            r2 = ses.solve(s)
        tuned = api.autotune_entries()
        assert tuned, "no product was large enough to tune"
        assert {t["kind"] for t in tuned} <= {"fp64_gemm_tile_ksplit", "split_gemm_kernel_raster"}
        for t in tuned:
            assert 0 <= t["choice"] < t["ncand"] and t["best_ms"] <= t["heuristic_ms"] + 1e-6
        assert r1.total_energy == r2.total_energy     # tuned choices are reused
        assert abs(r1.total_energy - ref.total_energy) <= 1e-11
        for k in ref.e2:
            assert abs(r1.e2[k] - ref.e2[k]) <= 1e-11
        api.autotune_mode(2)
        assert api.autotune_entries() == []
    finally:
        api.autotune_mode(prev)
