"""GPU DDM-3D (SOLVE_DDM3D_CHEM on the generated sparse LU) against the oracle's
restatement (dense LU with partial pivoting, FP64) for one CHEM call.

Tolerance: 1e-5 of each parameter's largest sensitivity (SENGRID is REAL(4); the two
sides factor the same matrix differently)."""
import numpy as np
import pytest

from helpers import gather_cells, to_cuda
from cmaq_gb300.synthetic import make_grid, manifest

pytestmark = pytest.mark.gpu

RTOL = float(np.float32(1e-3))
ATOL = float(np.float32(1e-9))


@pytest.mark.parametrize("mech", ["cb6r5_ae7_aq", "cracmm2"])
def test_ddm3d_matches_oracle(mech):
    import torch
    from oracle import Oracle, ddm3d_window
    from cmaq_gb300.chem import ChemSolver
    o = Oracle(mech)
    names = [sp["name"] for sp in manifest(mech)["species"]]
    g = make_grid(mech=mech, ncols=8, nrows=6, nlays=3, seed=81, het=True)
    y0, rki, night = gather_cells(g, o)
    i_o3, i_no2 = (int(o.iold2new[names.index(s)]) for s in ("O3", "NO2"))
    r_a, r_b = 0, 2
    params = [("init", i_o3), ("init", i_no2), ("rate", r_a), ("rate", r_b)]
    _, s_ref = ddm3d_window(o, y0, rki, night, 1, 5.0, RTOL, ATOL, params, threads=4)

    s = ChemSolver(mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd,
                   cgrid_index=g.cgrid_index, rtol=1e-3, atol=1e-9)
    t = to_cuda(g)
    npar = len(params)
    sen = torch.zeros((g.nspcsd, npar) + tuple(g.conc.shape[1:]), dtype=torch.float32, device="cuda")
    sen[g.cgrid_index[names.index("O3")] - 1, 0] = 1.0
    sen[g.cgrid_index[names.index("NO2")] - 1, 1] = 1.0
    mask = torch.zeros((npar, o.nrxns), dtype=torch.uint8, device="cuda")
    mask[2, r_a] = 1
    mask[3, r_b] = 1
    st = s.step_ddm(sen, *[t[k] for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj",
                                          "khetero")], rate_mask=mask)
    assert st["failed_cells"] == 0
    got = sen.cpu().numpy().reshape(g.nspcsd, npar, -1)
    for p in range(npar):
        ref = s_ref[p]                                          # [nspec solver order, n]
        gp = np.stack([got[g.cgrid_index[o.inew2old[i]] - 1, p] for i in range(o.nspec)])
        scale = np.abs(ref).max()
        assert np.abs(gp - ref).max() <= 1e-5 * scale, (p, np.abs(gp - ref).max() / scale)


def test_ddm3d_leaves_concentrations_as_plain_chem():
    from helpers import gpu_chem
    import torch
    g = make_grid(ncols=6, nrows=5, nlays=2, seed=82)
    plain, _, _ = gpu_chem(g, schedule="queue")
    from cmaq_gb300.chem import ChemSolver
    s = ChemSolver(g.mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd,
                   cgrid_index=g.cgrid_index, rtol=1e-3, atol=1e-9)
    t = to_cuda(g)
    sen = torch.zeros((g.nspcsd, 1) + tuple(g.conc.shape[1:]), dtype=torch.float32, device="cuda")
    s.step_ddm(sen, *[t[k] for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj",
                                     "khetero")])
    assert np.array_equal(t["conc"].cpu().numpy(), plain)
    assert float(sen.abs().max()) == 0.0


@pytest.mark.parametrize("mech", ["cb6r5_ae7_aq", "cracmm2"])
def test_ddm3d_with_smvgear_matches_oracle(mech):
    """The DDM-3D step of a Gear CHEM call (CAVEG from the Gear kernel) against the oracle's
    DDM-3D on SMVGEAR, both on the device's rate constants (SMVGEAR's discrete choices flip
    on ulp differences of exp/pow); tolerance as above."""
    import torch
    from oracle import Oracle, ddm3d_window
    from cmaq_gb300.chem import ChemSolver
    o = Oracle(mech)
    names = [sp["name"] for sp in manifest(mech)["species"]]
    g = make_grid(mech=mech, ncols=8, nrows=6, nlays=3, seed=84, het=True)
    s = ChemSolver(mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd,
                   cgrid_index=g.cgrid_index, rtol=1e-3, atol=1e-9, solver="gear")
    t = to_cuda(g)
    args = [t[k] for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj", "khetero")]
    rk_dev, _ = s.rconst(*args)
    y0, _, night = gather_cells(g, o, gear=True)
    i_o3, i_no2 = (int(o.iold2new[names.index(sp)]) for sp in ("O3", "NO2"))
    r_a, r_b = 0, 2
    params = [("init", i_o3), ("init", i_no2), ("rate", r_a), ("rate", r_b)]
    _, s_ref = ddm3d_window(o, y0, rk_dev.cpu().numpy(), night, 1, 5.0, RTOL, ATOL, params, threads=4,
                            gear_cfg=o.gear_cfg())
    npar = len(params)
    sen = torch.zeros((g.nspcsd, npar) + tuple(g.conc.shape[1:]), dtype=torch.float32, device="cuda")
    sen[g.cgrid_index[names.index("O3")] - 1, 0] = 1.0
    sen[g.cgrid_index[names.index("NO2")] - 1, 1] = 1.0
    mask = torch.zeros((npar, o.nrxns), dtype=torch.uint8, device="cuda")
    mask[2, r_a] = 1
    mask[3, r_b] = 1
    st = s.step_ddm(sen, *args, rate_mask=mask)
    assert st["failed_cells"] == 0
    got = sen.cpu().numpy().reshape(g.nspcsd, npar, -1)
    for p in range(npar):
        ref = s_ref[p]
        gp = np.stack([got[g.cgrid_index[o.inew2old[i]] - 1, p] for i in range(o.nspec)])
        scale = np.abs(ref).max()
        assert np.abs(gp - ref).max() <= 1e-5 * scale, (p, np.abs(gp - ref).max() / scale)


@pytest.mark.parametrize("mech", ["cb6r5_ae7_aq", "cracmm2"])
def test_ddm3d_with_ebi_matches_oracle(mech):
    """The DDM-3D step of an EBI CHEM call (YCDDM from the EBI kernels) against the oracle's
    DDM-3D on HRSOLVER with the EBI driver's gather.  Device and host rate constants differ
    by ulps (exp/pow), which can move EBI's convergence test in single cells: tolerance 1e-4
    of each parameter's largest sensitivity."""
    import torch
    from oracle import Oracle, ddm3d_window
    from cmaq_gb300.chem import ChemSolver
    o = Oracle(mech)
    names = [sp["name"] for sp in manifest(mech)["species"]]
    g = make_grid(mech=mech, ncols=8, nrows=6, nlays=3, seed=86, het=True)
    yc, rk, night = o.ebi_gather(g)
    y0 = yc[o.inew2old]
    i_o3, i_no2 = (int(o.iold2new[names.index(sp)]) for sp in ("O3", "NO2"))
    r_a, r_b = 0, 2
    params = [("init", i_o3), ("init", i_no2), ("rate", r_a), ("rate", r_b)]
    _, s_ref = ddm3d_window(o, y0, rk, night, 1, 5.0, RTOL, ATOL, params, threads=4, ebi=True)
    s = ChemSolver(mech, ncols=g.ncols, nrows=g.nrows, nlays=g.nlays, nspcsd=g.nspcsd,
                   cgrid_index=g.cgrid_index, rtol=1e-3, atol=1e-9, solver="ebi")
    t = to_cuda(g)
    npar = len(params)
    sen = torch.zeros((g.nspcsd, npar) + tuple(g.conc.shape[1:]), dtype=torch.float32, device="cuda")
    sen[g.cgrid_index[names.index("O3")] - 1, 0] = 1.0
    sen[g.cgrid_index[names.index("NO2")] - 1, 1] = 1.0
    mask = torch.zeros((npar, o.nrxns), dtype=torch.uint8, device="cuda")
    mask[2, r_a] = 1
    mask[3, r_b] = 1
    st = s.step_ddm(sen, *[t[k] for k in ("conc", "ta", "qv", "dens", "pres", "seaice", "ocean_szone", "rj",
                                          "khetero")], rate_mask=mask)
    assert st["failed_cells"] == 0
    got = sen.cpu().numpy().reshape(g.nspcsd, npar, -1)
    for p in range(npar):
        ref = s_ref[p]
        gp = np.stack([got[g.cgrid_index[o.inew2old[i]] - 1, p] for i in range(o.nspec)])
        scale = np.abs(ref).max()
        assert np.abs(gp - ref).max() <= 1e-4 * scale, (p, np.abs(gp - ref).max() / scale)
