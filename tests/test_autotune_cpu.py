"""Host-side logic of the autotuner (no GPU): the candidate space and the cache key."""
from cmaq_gb300.autotune import Candidate, cache_key, candidates


def test_candidate_space():
    c = candidates(("default", "r168"))
    assert len(c) == 2 * 7
    assert len(candidates()) == 6 * 7
    assert Candidate("default", 0, 8) in c                  # free-running warps only with 8-warp blocks
    assert all(x.block_warps in (2, 4, 8) and x.lockstep in (0, 1, 2) for x in c)
    assert not any(x.lockstep == 0 and x.block_warps != 8 for x in c)
    # block size is applied before the barrier granularity (every pair is reachable)
    assert list(Candidate("default", 0, 8).knobs()) == ["block_warps", "lockstep"]


def test_cache_key_buckets_grid_sizes():
    assert cache_key("cb6r5_ae7_aq", 4_803_435) == cache_key("cb6r5_ae7_aq", 4_500_000)
    assert cache_key("cb6r5_ae7_aq", 4_803_435) != cache_key("cb6r5_ae7_aq", 350_000)
    assert cache_key("cb6r5_ae7_aq", 1000) != cache_key("cracmm2", 1000)
