"""CPU oracle (ROS3 restatement): closed-form cases, invariants and semantics.

The reference ships no golden vectors for this path and cannot be compiled here
(Fortran), so the oracle is pinned by cases with known answers:
* a single first-order decay, against the exact exponential;
* the O3-NO-NO2 photostationary box, whose linear invariants (NOx, Ox) a
  Rosenbrock method preserves to round-off;
* a dark NO2 + NO3 <-> N2O5 box, which must relax to the thermal equilibrium;
and by the reference's own solver semantics (day/night lists, block step size).
"""
import numpy as np
import pytest

from cmaq_gb300.synthetic import make_grid, manifest

MECH = "cb6r5_ae7_aq"


@pytest.fixture(scope="module")
def o():
    from oracle import Oracle
    return Oracle(MECH)


@pytest.fixture(scope="module")
def man():
    return manifest(MECH)


def _idx(man, o, name):
    old = [s["name"] for s in man["species"]].index(name)
    return int(o.iold2new[old])


def _rx(man, label):
    return [r["label"] for r in man["reactions"]].index(label)


def _base_state(o, floor=1e-30):
    return np.full((o.nspec, 1), floor)


def test_first_order_decay_matches_exponential(o, man):
    # R21: H2O2 -> 2 OH (photolysis); every other rate constant zero
    r = _rx(man, "R21")
    assert man["reactions"][r]["nreact"] == 1
    k = np.zeros((o.nrxns, 1))
    k[r] = 0.2                      # 1/min
    y = _base_state(o)
    ih, ioh = _idx(man, o, "H2O2"), _idx(man, o, "OH")
    y[ih] = 1.0e-3
    yt, st = o.solve_block(y, k, 0, 5.0, 1e-8, 1e-20)
    assert st[3] == 0
    exact = 1.0e-3 * np.exp(-0.2 * 5.0)
    assert abs(yt[ih, 0] - exact) / exact < 1e-6
    assert abs(yt[ioh, 0] - 2.0 * (1.0e-3 - exact)) / (2e-3) < 1e-6


def test_photostationary_box_keeps_linear_invariants(o, man):
    # R1 NO2 -> NO + O, R2 O + O2 (+M) -> O3, R3 O3 + NO -> NO2
    rs = [_rx(man, lab) for lab in ("R1", "R2", "R3")]
    k = np.zeros((o.nrxns, 1))
    k[rs[0]] = 0.5
    k[rs[1]] = 5.0e5                # fast O recombination (pseudo-first order)
    k[rs[2]] = 26.0                 # 1/(ppm min)
    y = _base_state(o)
    ino, ino2, io3, iox = (_idx(man, o, s) for s in ("NO", "NO2", "O3", "O"))
    y[ino], y[ino2], y[io3] = 0.01, 0.02, 0.04
    yt, st = o.solve_block(y, k, 0, 5.0, 1e-3, 1e-12)
    assert st[3] == 0
    nox0, ox0 = y[ino] + y[ino2], y[io3] + y[ino2] + y[iox]
    assert abs((yt[ino] + yt[ino2]) - nox0)[0] / nox0[0] < 1e-12
    assert abs((yt[io3] + yt[ino2] + yt[iox]) - ox0)[0] / ox0[0] < 1e-12
    # after 5 min (relaxation time ~ 1/(J + k3 (O3 + NO)) ~ 0.6 min) the box is photostationary
    pss = 0.5 * yt[ino2, 0] / (26.0 * yt[io3, 0] * yt[ino, 0])
    assert abs(pss - 1.0) < 1e-2


def test_dark_n2o5_equilibrium(o, man):
    # R17 NO2 + NO3 -> N2O5 (falloff), R18? thermal decomposition N2O5 -> NO2 + NO3
    labels = [r["label"] for r in man["reactions"]]
    ino2, ino3, in2o5 = (_idx(man, o, s) for s in ("NO2", "NO3", "N2O5"))
    fwd = rev = None
    for r, rx in enumerate(man["reactions"]):
        names_r = sorted(man["species"][s]["name"] for s in rx["reactants"])
        names_p = sorted(man["species"][s]["name"] for s in rx["products"])
        if names_r == ["NO2", "NO3"] and names_p == ["N2O5"]:
            fwd = r
        if names_r == ["N2O5"] and names_p == ["NO2", "NO3"] and not rx["photolytic"]:
            rev = r
    assert fwd is not None and rev is not None, labels[:5]
    k = np.zeros((o.nrxns, 1))
    k[fwd], k[rev] = 2.0e3, 3.0            # 1/(ppm min), 1/min
    y = _base_state(o)
    y[ino2], y[ino3], y[in2o5] = 0.01, 5.0e-4, 1.0e-5
    yt, st = o.solve_block(y, k, 1, 5.0, 1e-6, 1e-14)
    assert st[3] == 0
    ratio = yt[in2o5, 0] / (yt[ino2, 0] * yt[ino3, 0])
    assert abs(ratio / (2.0e3 / 3.0) - 1.0) < 1e-4
    tot_n = yt[ino2] + yt[ino3] + 2 * yt[in2o5]
    assert abs(tot_n - (y[ino2] + y[ino3] + 2 * y[in2o5]))[0] < 1e-14


def test_dark_cells_get_no_photolysis(o, man):
    n = 4
    k = o.rconst(np.full(n, 280.0), np.full(n, 1.0), np.full(n, 1e4), np.full((o.nphotab, n), 0.01),
                 np.zeros((o.nhetero, n)), False, np.full(n, 0.5))
    blocks = man["rate_tables"]["rate_block"]
    photo = [int(r) for r, b in blocks.items() if b != "thermal"]
    assert np.all(k[photo] == 0.0)
    assert np.all(k[[int(r) for r, b in blocks.items() if b == "thermal"]] >= 0.0)


def test_seawater_halogen_rate_only_above_threshold(o, man):
    r = [int(x) for x, b in man["rate_tables"]["rate_block"].items() if b == "seawater"][0]
    k = o.rconst(np.full(3, 290.0), np.full(3, 1.0), np.full(3, 1e4), np.full((o.nphotab, 3), 0.01),
                 np.zeros((o.nhetero, 3)), True, np.array([0.0, 0.001, 0.5]))
    assert k[r, 0] == 0.0 and k[r, 1] == 0.0 and k[r, 2] > 0.0


def test_chem_is_deterministic_across_threads(o):
    g = make_grid(ncols=8, nrows=5, nlays=3, seed=4)
    a, ta = o.chem(g, blksize=50, threads=1)
    b, tb = o.chem(g, blksize=50, threads=4)
    assert np.array_equal(a, b) and ta == tb


def test_block_and_cell_semantics_agree_with_tight_solution(o):
    g = make_grid(ncols=6, nrows=5, nlays=2, seed=9)
    rt, at = float(np.float32(1e-3)), float(np.float32(1e-9))
    blk, _ = o.chem(g, blksize=50, rtol=rt, atol=at)
    cell, _ = o.chem(g, blksize=1, rtol=rt, atol=at)
    with o.tight():
        tight, st = o.chem(g, blksize=1, rtol=1e-8, atol=1e-14)
    assert st["rc"] == 0
    m = tight > 1e-6
    e_blk = np.max(np.abs(blk[m] - tight[m]) / tight[m])
    e_cell = np.max(np.abs(cell[m] - tight[m]) / tight[m])
    assert e_blk < 0.05 and e_cell < 0.05
    assert not np.array_equal(blk, cell)   # the shared block step size changes the numbers


def test_reordering_pass_changes_only_block_membership(o):
    g = make_grid(ncols=10, nrows=10, nlays=2, seed=12)
    a, _ = o.chem(g, blksize=50, lreorder=True)
    b, _ = o.chem(g, blksize=50, lreorder=False)
    c1, _ = o.chem(g, blksize=1, lreorder=True)
    c2, _ = o.chem(g, blksize=1, lreorder=False)
    assert np.array_equal(c1, c2)          # per-cell integration does not depend on the order
    assert np.isfinite(a).all() and np.isfinite(b).all()
