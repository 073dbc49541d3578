"""Autotuner plan and cache logic (no GPU): gbjk_tune_plan's rules and
overrides, and the text cache of tuned launch choices."""
import pytest

from chem_gb300.fock import k_split_plan, tune_cache_lookup, tune_cache_store, tune_plan


@pytest.mark.parametrize("nbf,naux,nocc", [(24, 116, 5), (130, 510, 17), (490, 2366, 81),
                                           (800, 2400, 120)])
def test_rules_match_the_published_plan(nbf, naux, nocc):
    eff, ks = tune_plan(nbf, naux, nocc)
    assert (ks, eff["fp64_kchunk"]) == k_split_plan(nbf, naux, nocc)
    assert eff["fp64_ht_tn"] in (1, 16, 32, 64) and eff["fp64_k_tile"] in (1, 64)
    # the rules: one thread per output below 2^20 outputs, 64 x 32 tiles
    # when nocc pads better to 32 than to 64
    if nbf * naux * nocc <= 1 << 20:
        assert eff["fp64_ht_tn"] == 1
    if (nbf, nocc) == (490, 81):
        assert eff["fp64_ht_tn"] == 32


def test_overrides_round_and_cover_the_sum():
    nbf, naux, nocc = 490, 2366, 81
    kdim = naux * nocc
    for req in (1, 100, 1000, 50000, 10 ** 9):
        eff, ks = tune_plan(nbf, naux, nocc, fp64_kchunk=req)
        kc = eff["fp64_kchunk"]
        assert kc % 16 == 0 and kc >= 16
        assert (ks - 1) * kc < kdim <= ks * kc
    eff, _ = tune_plan(nbf, naux, nocc, fp64_ht_tn=16, fp64_k_tile=1)
    assert eff["fp64_ht_tn"] == 16 and eff["fp64_k_tile"] == 1
    for bad in ({"fp64_ht_tn": 8}, {"fp64_k_tile": 32}, {"fp64_kchunk": -1}):
        with pytest.raises(RuntimeError):
            tune_plan(nbf, naux, nocc, **bad)


def test_cache_last_line_wins(tmp_path):
    path = str(tmp_path / "tune.txt")
    assert tune_cache_lookup(path, "sigA") is None  # no file
    tune_cache_store(path, "sigA", fp64_ht_tn=32, fp64_k_tile=64, fp64_kchunk=4000)
    tune_cache_store(path, "sigB", split_ksplit=7, overlap_sms=8)
    assert tune_cache_lookup(path, "sigA")["fp64_kchunk"] == 4000
    tune_cache_store(path, "sigA", fp64_ht_tn=16, fp64_kchunk=8000)
    got = tune_cache_lookup(path, "sigA")
    assert got["fp64_ht_tn"] == 16 and got["fp64_kchunk"] == 8000
    assert tune_cache_lookup(path, "sigB") == {"fp64_ht_tn": 0, "fp64_k_tile": 0,
                                               "fp64_kchunk": 0, "split_ksplit": 7,
                                               "overlap_sms": 8}
    assert tune_cache_lookup(path, "sigC") is None
    with pytest.raises(RuntimeError):
        tune_cache_store(path, "bad signature", fp64_ht_tn=16)
