"""GPU parity of the heterogeneous rate constants (HETCHEM_RATES, CCTM/src/aero/aero6/
AEROSOL_CHEMISTRY.F) against the oracle, through the C ABI
(cmaqchem_hetchem_rates_device, cmaqchem_hetchem_rates).

The device code performs the oracle's IEEE operations in the same order (built with
-fmad=false), but its exp, log, pow, tanh and log10 (float and double) are CUDA's, which
differ from the host library's by an ulp or two.  The outputs are smooth functions of
those values with no step-size amplification, so the bar is a relative difference of
1e-5 per KHETERO entry (float intermediates carry 6e-8 per ulp) — except where the
reference's own arithmetic is ill-conditioned: CALCISOPGAMMAS forms the IEPOX uptake
coefficient from q / TANH( q ) - 1 (AEROSOL_CHEMISTRY.F:2517-2526), about q^2 / 3, a
difference of two numbers next to 1, so an ulp of TANH moves IEPOX, IEPOXOS and TETROL
(CRACMM2: ISO3NOSJ, ISO3OSJ) by up to 2^-52 / (q^2 / 3) relative, and for q below about
2e-7 decides whether they are zero at all (the switch q / TANH( q ) > 1).  Those labels
are held to that bound with the oracle's q of each cell.  N2O5_GAMMA's coarse-mode
(Bertram and Thornton) form has the same kind of term in REAL(4): k2f = beta - beta
EXP( -delta [H2O] ) (AEROSOL_CHEMISTRY.F:1937), whose relative error from an ulp of EXP
is 2^-24 / (delta [H2O]) for a dry coarse mode; HETERO_N2O5K is held to that bound.
Every other entry must meet 1e-5.
tests/test_hetchem_host.py holds the same code, built for the host, to the oracle bit
for bit.
"""
import numpy as np
import pytest

h = pytest.importorskip("hetchem")   # oracle/hetchem.py
pytestmark = pytest.mark.gpu
RTOL = 1e-5


def _dev(*arrays):
    import torch
    return [torch.from_numpy(np.ascontiguousarray(a)).cuda() for a in arrays]


# the labels formed from CALCISOPGAMMAS' uptake coefficient and product fractions
IEPOX_FAMILY = ("HETERO_IEPOX", "HETERO_IEPOXOS", "HETERO_TETROL", "HETERO_ISO3NOSJ", "HETERO_ISO3OSJ")


@pytest.mark.parametrize("mech", ["cb6r5_ae7_aq", "cracmm2"])
def test_layout_matches_the_tables(mech):
    from cmaq_gb300.hetchem import layout
    t = h.tables(mech)
    assert layout(mech) == (len(t["ae_rows"]), t["ae_first"], len(t["hetero"]))
    from cmaq_gb300 import _lib
    with pytest.raises(_lib.ChemError):
        layout("saprc07tc_ae6_aq")


@pytest.mark.parametrize("mech,n,seed", [("cb6r5_ae7_aq", 20000, 21), ("cb6r5_ae7_aq", 777, 4),
                                         ("cracmm2", 20000, 22)])
def test_device_rates_match_the_oracle(mech, n, seed):
    import torch
    from cmaq_gb300.hetchem import hetchem_rates
    from cmaq_gb300.synthetic import make_aerosol_cells
    ae, ta, p, q, d = make_aerosol_cells(n, seed=seed, mech=mech)
    got = hetchem_rates(*_dev(ae, ta, p, q, d), mechanism=mech)
    torch.cuda.synchronize()
    got = got.cpu().numpy()
    want = h.rates(ae, ta, p, q, d, threads=8, mech=mech)
    assert np.isfinite(got).all()
    t = h.tables(mech)
    switch = [j for j, x in enumerate(t["hetero"]) if x in IEPOX_FAMILY]
    rel = np.where(got == want, 0.0, np.abs(got - want) / np.maximum(np.abs(want), 1e-300))
    bad = rel > RTOL
    bad[:, switch] = False
    jk = t["hetero"].index("HETERO_N2O5K") if "HETERO_N2O5K" in t["hetero"] else None
    for c in (np.nonzero(bad[:, jk])[0] if jk is not None else []):   # the coarse-mode gamma's conditioning
        _, m3, _ = h.cell_piece("moments", ae[:, c], mech=mech)
        mw = {s_["bulkname"]: np.float32(s_["molwt"]) for s_ in t["species"]}
        inv_vol = np.float32(1e-9) * (np.float32(6.0) / np.float32(3.14159265)) / np.float32(m3[2])
        rows = {nm: i for i, nm in enumerate(t["ae_rows"])}
        ah2om = max(ae[rows["AH2OK"], c], np.float32(1e-23)) * inv_vol / mw["AH2O"]
        x = float(np.float32(0.13) * ah2om)
        if rel[c, jk] <= RTOL + 8.0 * 2.0 ** -24 / x:
            bad[c, jk] = False
    assert not bad.any(), [(int(c), t["hetero"][j], got[c, j], want[c, j]) for c, j in np.argwhere(bad)[:8]]
    qs = np.array([h.cell_piece("isop_q", ae[:, c], float(ta[c]), mech=mech) for c in range(n)])
    cond = np.maximum(qs * qs / 3.0, 1e-300)            # q / tanh(q) - 1
    eps = 2.0 ** -52
    allowed = RTOL + 16.0 * eps / cond
    flip = (got[:, switch] == 0) != (want[:, switch] == 0)
    assert (~flip.any(axis=1) | (cond < 64.0 * eps)).all(), qs[flip.any(axis=1)][:5]
    rs = np.where(flip, 0.0, rel[:, switch])
    worst = (rs / allowed[:, None]).max()
    assert worst <= 1.0, worst
    print(f"{mech}: {int(flip.any(axis=1).sum())} of {n} cells on the q / TANH( q ) switch; "
          f"IEPOX-family error at most {worst:.2f} of its conditioning bound")


@pytest.mark.parametrize("mech", ["cb6r5_ae7_aq", "cracmm2"])
def test_cgrid_view_and_host_entry_give_the_same_bits(mech):
    """The aerosol block read in place from a CGRID (CONC(1,1,1,AE_STRT) with the gas rows
    before it), and the host-array entry, equal the compact device call bit for bit."""
    import torch
    from cmaq_gb300.hetchem import hetchem_rates, hetchem_rates_host, layout
    from cmaq_gb300.synthetic import make_aerosol_cells
    nae, first, _ = layout(mech)
    ae, ta, p, q, d = make_aerosol_cells(5000, seed=8, mech=mech)
    cgrid = np.full((first + nae + 3, ae.shape[1]), -1.0, np.float32)
    cgrid[first:first + nae] = ae
    cg, tt, pt, qt, dt = _dev(cgrid, ta, p, q, d)
    a = hetchem_rates(cg[first:first + nae], tt, pt, qt, dt, mechanism=mech).cpu().numpy()
    b = hetchem_rates(*_dev(ae), tt, pt, qt, dt, mechanism=mech).cpu().numpy()
    c = hetchem_rates_host(ae, ta, p, q, d, mechanism=mech)
    torch.cuda.synchronize()
    assert np.array_equal(a, b) and np.array_equal(b, c)


def test_empty_call_and_bad_arguments():
    from cmaq_gb300 import _lib
    L = _lib.lib()
    assert L.cmaqchem_hetchem_rates_device(b"cb6r5_ae7_aq", 0, None, None, None, None, None, None, None) == 0
    assert L.cmaqchem_hetchem_rates_device(b"cb6r5_ae7_aq", 5, None, None, None, None, None, None, None) == -1
    assert "null" in _lib.last_error()
