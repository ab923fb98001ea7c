"""Per-file compile flags of the library's build variants (cmaq_gb300/build.py)."""
from cmaq_gb300 import build as b


def _flags(name, variant):
    src = b.CSRC / name
    gen_extra, all_extra = (list(x) for x in b.VARIANTS[variant])
    return b._flags(src, variant, gen_extra, all_extra)


def test_kmt2_switches_reach_kmt2_only():
    for v in ("kq2", "kq3", "kqfree", "kqr1", "kqr8", "kqr32"):
        assert any(f.startswith("-DKMT2_") for f in _flags("kmt2.cu", v))
        for name in ("chem_capi.cu", "gen/cb6r5_ae7_aq_rates.cu", "gen/cracmm2_rates.cu", "hetchem.cu"):
            assert _flags(name, v) == _flags(name, "default"), (v, name)


def test_default_exceptions():
    assert _flags("gen/cracmm2_rates.cu", "default") == [b.Q16] + b.GEN128
    assert _flags("gen/cb6r5_ae7_aq_rates.cu", "default") == [b.Q_DEFAULT] + b.GEN_DEFAULT
    assert _flags("chem_capi.cu", "w16") == [b.Q16]
