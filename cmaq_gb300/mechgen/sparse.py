"""Symbolic sparse structure of the ROS3 iteration matrix.

Restates the symbolic part of CMAQ's ROS3 solver set-up
(CCTM/src/gas/ros3/rbsparse.F) so that the oracle and the generated device code
use exactly the reference's species order, active-reaction lists, LU fill
pattern, storage order and operation order:

* species reorder, fewest partial-derivative terms first, non-reacting species
  last, by the same selection sort (rbsparse.F:208-252);
* day / night active reactions: a reaction with ``BTEST(IRXBITS, 1)`` (a
  photolysis reaction) is dropped at night; reactions without reactants are
  never active (rbsparse.F:259-281);
* symbolic Doolittle LU column by column, recording each
  ``A(i,j) -= A(i,k) * A(k,j)`` update and each ``A(i,j) *= 1/A(j,j)``
  scaling in the reference's order (rbsparse.F:385-421);
* storage index ``JARRAYPT``: strictly-lower entries row by row, then
  strictly-upper entries from the last row upwards, then the diagonal
  (rbsparse.F:426-460);
* partial-derivative scatter lists ``JARRL/JLIAL`` and ``JARRP/JPIAL/ICOEFF``
  (rbsparse.F:614-646).

Storage indices here are 1-based like the reference's ``CC2(:, 0:IARRAY)``;
slot 0 is the reference's scratch slot that is zeroed but never referenced by
a valid entry.
"""
from __future__ import annotations

from dataclasses import dataclass, field

from .fortran_tables import Mechanism


@dataclass
class SparseMech:
    ischan: int
    inew2old: list[int]                 # new (0-based) -> old (0-based)
    iold2new: list[int]
    irm2: list[list[int]]               # [rxn][0..2 reactants, 3.. products] new 0-based index, -1 none
    active: list[list[int]]             # [ncsp][...] 0-based reactions
    iarray: list[int]                   # [ncsp] number of stored LU entries
    jarraypt: list[dict]                # [ncsp] {(i,j) new 0-based -> storage index 1-based}
    decomp_ops: list[list[list[tuple[int, int, int]]]]   # [ncsp][col j] -> [(ij, ik, kj)]
    lscale: list[list[list[int]]]       # [ncsp][col j] -> [ij] entries scaled by vdiag(j)
    diag: list[list[int]]               # [ncsp][i] storage index of (i,i)
    lower: list[list[list[tuple[int, int]]]]  # [ncsp][row i] -> [(storage, col j)] j<i ascending
    upper: list[list[list[tuple[int, int]]]]  # [ncsp][row i] -> [(storage, col j)] j>i ascending
    loss_pd: list[dict]                 # [ncsp] {rxn: [(storage, ial)]}
    prod_pd: list[dict]                 # [ncsp] {rxn: [(storage, ial, icoeff)]}  icoeff: -1 unit, else product slot
    nnz_jac: list[int] = field(default_factory=list)


def build_sparse(mech: Mechanism) -> SparseMech:
    ns, nr = mech.nspec, mech.nrxns
    irr = mech.irr
    # --- partial-derivative pattern in old species order (rbsparse.F:173-191)
    isparder = [[0] * ns for _ in range(ns)]     # [iporr][ireact]
    for r in range(nr):
        for k in range(3):
            ire = irr[r][k]
            if ire != 0:
                for kk in range(3 + mech.mxprd):
                    ip = irr[r][kk]
                    if ip != 0:
                        isparder[ip - 1][ire - 1] = 1
    isaporl = [sum(isparder[i][j] for j in range(ns)) for i in range(ns)]

    # --- reacting species first, non-reacting at the bottom (rbsparse.F:199-210)
    inew2old = [0] * ns
    iold2new = [0] * ns
    ischan = 0
    nochang = ns - 1
    for jold in range(ns):
        if isaporl[jold] > 0:
            inew2old[ischan] = jold
            iold2new[jold] = ischan
            ischan += 1
        else:
            inew2old[nochang] = jold
            iold2new[jold] = nochang
            nochang -= 1
    # --- selection sort by number of PD terms (rbsparse.F:216-252)
    for jnew in range(ischan):
        jold = inew2old[jnew]
        minvalu = isaporl[jold]
        iminold, iminnew = jold, jnew
        for inew in range(jnew + 1, ischan):
            iold = inew2old[inew]
            if isaporl[iold] < minvalu:
                minvalu = isaporl[iold]
                iminold, iminnew = iold, inew
        inew2old[iminnew] = jold
        inew2old[jnew] = iminold
        iold2new[jold] = iminnew
        iold2new[iminold] = jnew

    # --- IRM2 and active lists (rbsparse.F:259-281)
    irm2 = [[-1] * (3 + mech.mxprd) for _ in range(nr)]
    active = [[], []]
    for r in range(nr):
        for k in range(mech.nreact[r]):
            irm2[r][k] = iold2new[irr[r][k] - 1]
        for p in range(mech.nprdct[r]):
            irm2[r][3 + p] = iold2new[irr[r][3 + p] - 1]
        if mech.nreact[r] > 0:
            active[0].append(r)
            if not (mech.irxbits[r] >> 1) & 1:
                active[1].append(r)

    res = SparseMech(ischan=ischan, inew2old=inew2old, iold2new=iold2new, irm2=irm2, active=active,
                     iarray=[0, 0], jarraypt=[{}, {}], decomp_ops=[[], []], lscale=[[], []],
                     diag=[[], []], lower=[[], []], upper=[[], []], loss_pd=[{}, {}], prod_pd=[{}, {}])
    n = ischan
    for ncsp in range(2):
        # symbolic Jacobian, LZERO(row, col) (rbsparse.F:327-344)
        lz = [[0] * ns for _ in range(ns)]
        for i in range(ns):
            lz[i][i] = 1
        for r in active[ncsp]:
            for k in range(mech.nreact[r]):
                ire = irm2[r][k]
                for jal in range(mech.nreact[r]):
                    lz[irm2[r][jal]][ire] = 1
                for p in range(mech.nprdct[r]):
                    lz[irm2[r][3 + p]][ire] = 1
        res.nnz_jac.append(sum(lz[i][j] for i in range(n) for j in range(n)))
        # symbolic decomposition (rbsparse.F:385-421)
        ops_sym: list[list[tuple[int, int]]] = []     # per column j: [(i, k)]
        lsc_sym: list[list[int]] = []                 # per column j: [i]
        for j in range(n):
            colops = []
            for i in range(1, n):
                kmax = min(i, j)                  # K = 1..min(I-1, J-1), 1-based
                for k in range(kmax):
                    if lz[i][k] == 1 and lz[k][j] == 1:
                        colops.append((i, k))
                        lz[i][j] = 1
            ops_sym.append(colops)
            lsc_sym.append([i for i in range(j + 1, n) if lz[i][j] == 1])
        # storage order (rbsparse.F:426-460)
        jpt: dict[tuple[int, int], int] = {}
        cnt = 0
        lower = [[] for _ in range(n)]
        upper = [[] for _ in range(n)]
        for i in range(1, n):
            for j in range(i):
                if lz[i][j] == 1:
                    cnt += 1
                    jpt[(i, j)] = cnt
                    lower[i].append((cnt, j))
        for i in range(n - 2, -1, -1):
            for j in range(i + 1, n):
                if lz[i][j] == 1:
                    cnt += 1
                    jpt[(i, j)] = cnt
                    upper[i].append((cnt, j))
        diag = []
        for i in range(n):
            cnt += 1
            jpt[(i, i)] = cnt
            diag.append(cnt)
        res.iarray[ncsp] = cnt
        res.jarraypt[ncsp] = jpt
        res.lower[ncsp] = lower
        res.upper[ncsp] = upper
        res.diag[ncsp] = diag
        res.decomp_ops[ncsp] = [[(jpt[(i, j)], jpt[(i, k)], jpt[(k, j)]) for (i, k) in ops_sym[j]]
                                for j in range(n)]
        res.lscale[ncsp] = [[jpt[(i, j)] for i in lsc_sym[j]] for j in range(n)]
        # PD scatter lists (rbsparse.F:614-646)
        lpd, ppd = {}, {}
        for r in active[ncsp]:
            ll, pp = [], []
            for ial in range(mech.nreact[r]):
                ir = irm2[r][ial]
                for jal in range(mech.nreact[r]):
                    jr = irm2[r][jal]
                    ll.append((jpt[(jr, ir)], ial))
                for iap in range(mech.nprdct[r]):
                    jp = irm2[r][3 + iap]
                    icoeff = iap if abs(mech.sc[r][iap] - 1.0) > 1.0e-6 else -1
                    pp.append((jpt[(jp, ir)], ial, icoeff))
            lpd[r] = ll
            ppd[r] = pp
        res.loss_pd[ncsp] = lpd
        res.prod_pd[ncsp] = ppd
    return res


def flop_counts(mech: Mechanism, sp: SparseMech, ncsp: int) -> dict[str, int]:
    """Algorithmic FLOPs of one ROS3 step per cell, counted on the reference's
    operations (a multiply-add counts 2, a divide or reciprocal counts 1)."""
    act = sp.active[ncsp]
    n = sp.ischan
    ns = mech.nspec
    fe = 0
    for r in act:
        nre = mech.nreact[r]
        fe += nre + nre + 2 * mech.nprdct[r]     # rate product, losses, SC * rate adds
    jac = 0
    for r in act:
        nre = mech.nreact[r]
        jac += {1: 0, 2: 2, 3: 5}.get(nre, 0)     # partial-derivative products
        jac += len(sp.loss_pd[ncsp][r])
        jac += sum(1 if ic < 0 else 2 for (_, _, ic) in sp.prod_pd[ncsp][r])
    nops = sum(len(c) for c in sp.decomp_ops[ncsp])
    nsc = sum(len(c) for c in sp.lscale[ncsp])
    lu = 2 * nops + nsc + n
    nl = sum(len(x) for x in sp.lower[ncsp])
    nu = sum(len(x) for x in sp.upper[ncsp])
    solve = 2 * (nl + nu) + n
    # diagonal shift; YP = Y + K1; K2 and K3 right-hand sides; YP = Y + sum(B K);
    # weighted error (3-term combination, tolerance, divide, square-accumulate); accept max
    vec = n + ns + 2 * ns + 4 * ns + 6 * ns + 10 * ns + ns
    total = 2 * fe + jac + lu + 3 * solve + vec
    return {"feval": fe, "jacobian": jac, "decomp": lu, "decomp_fma": nops, "decomp_scale": nsc,
            "solve": solve, "nnz_l": nl, "nnz_u": nu, "vector": vec, "step_total": total}
