"""CPU tests of the oracle's global thermodynamic observables (ThermoCalculator::compute,
thermo/ThermoCalculator.h:68-90): against a direct numpy restatement over all pairs, the
existing global virial, and the symmetries of the Born tensor."""
import numpy as np
import pytest


def _direct(oracle, box, pos, diam, pot, vel, mass, disp, max_rc):
    """Every pair i < j within max_rcut, r_ij = r_i - r_j (min image), the reference's
    formulas (ListofCommonObservables.h), divided by the volume."""
    D = box.dim
    L = np.array([box.L[c] for c in range(3)])
    per = np.array([box.periodic[c] for c in range(3)], bool)
    n = len(pos)
    pe, vir, ela = 0.0, np.zeros((D, D)), np.zeros((D, D))
    born = np.zeros((D,) * 4)
    for i in range(n):
        for j in range(i + 1, n):
            r = pos[i] - pos[j]
            r = np.where(per, r - L * np.rint(r / L), r)
            rsq = float(r @ r)
            if not rsq < max_rc * max_rc:
                continue
            pe += oracle.pair_energy(pot, rsq, diam[i], diam[j])
            f = oracle.force_divr(pot, rsq, diam[i], diam[j])
            vir += f * np.outer(r[:D], r[:D])
            w = (disp[j] - disp[i]) + r
            f1 = oracle.force_divr(pot, float(w @ w), diam[i], diam[j])
            ela += f1 * np.outer(w[:D], w[:D]) - f * np.outer(r[:D], r[:D])
            s = oracle.bond_stiffness(pot, rsq, diam[i], diam[j])
            rr = r[:D]
            nn = rr / np.sqrt(rsq)
            born += np.einsum("i,j,k,l->ijkl", s * rr + f * rr, rr, nn, nn)
    kin = np.einsum("n,na,nb->ab", mass, vel[:, :D], vel[:, :D])
    vol = np.prod(L[:D])
    return {"potentialenergy": pe / vol, "virialstress": vir / vol, "elasticvirialstress": ela / vol,
            "kineticstress": kin / vol, "borntensor": born / vol}


@pytest.mark.parametrize("kind,dim", [("poly12", 2), ("lj", 2), ("polyyukawa", 2), ("poly10", 3)])
def test_global_thermo_matches_direct_sum(oracle, kind, dim):
    from pyglasstools_gb300 import synth
    fr = synth.make_frame(150 if dim == 2 else 216, dim=dim, seed=5)
    if kind == "lj" or kind == "polyyukawa":  # long cut-offs: a larger box of the same density
        fr = synth.make_frame(400, dim=dim, seed=5)
    rc, prm = oracle.potential_params(kind)
    pot = oracle.make_potential(kind, rc, prm)
    box = oracle.make_box(dim, [fr.L, fr.L, fr.L if dim == 3 else 1.0])
    rng = np.random.default_rng(3)
    disp = np.zeros((len(fr.pos), 3))
    disp[:, :dim] = rng.normal(0, 0.02, (len(fr.pos), dim))
    max_rc = oracle.max_rcut(rc, fr.diam)
    got = oracle.global_thermo(box, fr.pos, fr.diam, pot, vel=fr.vel, mass=fr.mass, disp=disp, max_rc=max_rc)
    want = _direct(oracle, box, fr.pos, fr.diam, pot, fr.vel, fr.mass, disp, max_rc)
    for k, v in want.items():
        np.testing.assert_allclose(got[k], v, rtol=1e-12, atol=1e-12 * np.max(np.abs(v)), err_msg=k)
    assert abs(got["potentialenergy"]) > 0 and np.max(np.abs(got["borntensor"])) > 0
    # the pair virial as the existing global-virial routine has it (before the 1/vol)
    vol = fr.L ** dim
    np.testing.assert_allclose(got["virialstress"] * vol, oracle.global_virial(box, fr.pos, fr.diam, pot, max_rc),
                               rtol=1e-12, atol=1e-12)
    # Born: (s + f) r_i r_j r_k r_l / r^2 -- symmetric under any index swap
    b = got["borntensor"]
    for perm in [(1, 0, 2, 3), (0, 1, 3, 2), (2, 3, 0, 1), (0, 2, 1, 3)]:
        np.testing.assert_allclose(b, b.transpose(perm), rtol=1e-12, atol=1e-12 * np.max(np.abs(b)))
