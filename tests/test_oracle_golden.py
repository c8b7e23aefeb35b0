"""The FP64 CPU oracle against the reference's own golden vectors.

Fixtures (tests/golden/, extracted from the reference by make_golden.py):
  * Si.soap.cur_points.json  -- 100 SOAP vectors, reference tolerance 1e-8
    (tests/test_gapfit.py:58, config :93-95)
  * test_descriptor.py       -- C2H SOAP gradient values and index table, tol 1e-7
    (tests/test_descriptor.py:68-190, :211-226)
  * test_gappot.py           -- distance_2b GAP energy (1e-5) and forces (1e-6)
  * test_potential_cell.py   -- H2 in cells 2.5..4.5 A, cutoff 4 > cell, tol 1e-6
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle
from quip_gb300 import models
from quip_gb300.atoms import read_xyz

SI_SOAP = ("soap atom_sigma=0.5 central_weight=1.0 cutoff=4.0 cutoff_transition_width=1.0 "
           "l_max=8 n_max=8 n_species=1 species_Z={14} Z=14")


def test_si_soap_cur_points(golden):
    frames = read_xyz(os.path.join(golden, "Si.np1.xyz"))
    ref = np.load(os.path.join(golden, "si_soap_cur_points.npz"))
    X, idx = ref["sparsex"], ref["index"]
    assert X.shape == (100, 325)
    # global 1-based atom index -> (frame, atom)
    where = [(f, k) for f, fr in enumerate(frames) for k in range(len(fr))]
    assert len(where) == 439
    per_frame = {}
    for t, gi in enumerate(idx):
        f, k = where[gi - 1]
        per_frame.setdefault(f, []).append((t, k))
    worst = 0.0
    for f, items in per_frame.items():
        fr = frames[f]
        q = oracle.soap(SI_SOAP, fr.positions, fr.numbers, fr.lattice, fr.pbc)
        for t, k in items:
            worst = max(worst, np.abs(q[k] - X[t]).max())
    assert worst < 1e-8, worst


def test_c2h_soap_gradients(golden):
    ref = np.load(os.path.join(golden, "c2h_soap_grad.npz"))
    pos = np.array([[0., 0., 0.], [0.875, 0.875, 0.875], [0.2, 0.2, 0.1]])
    cell = np.array([[0.0, 1.75, 1.75], [1.75, 0.0, 1.75], [1.75, 1.75, 0.0]])
    Z = np.array([6, 6, 1])
    # quippy's Descriptor.calc builds the connection with cutoff = descriptor cutoff + 1
    q, g, gi = oracle.soap("soap cutoff=1.3 l_max=4 n_max=4 atom_sigma=0.5 n_Z=2 Z={1 6}", pos, Z, cell.T, [1, 1, 1],
                           grad=True, list_cutoff=2.3)
    assert q.shape == (3, 51)
    assert g.shape == (7, 3, 51)
    np.testing.assert_array_equal(gi, ref["grad_index"])
    assert np.abs(g[:2] - ref["grad"]).max() < 1e-7


def _water():
    return read_xyz(os.path.join(os.path.dirname(__file__), "golden", "gap_water", "gap_sample.xyz"))[0]


def test_gap_distance_2b_energy_forces(golden):
    at = _water()
    m = oracle.OracleModel.from_xml(os.path.join(golden, "gap_water", "GAP.xml"))
    r = m.calc(at.positions, at.numbers, at.lattice, [1, 1, 1])
    assert abs(r["energy"] - at.info["energy"]) < 1e-5
    assert np.abs(r["force"] - at.arrays["force"]).max() < 1e-6
    # tighter than the reference test: FP64 restatement of the same arithmetic
    assert abs(r["energy"] - at.info["energy"]) < 1e-7


def test_potential_cell_energies(golden):
    d = json.load(open(os.path.join(golden, "potential_cell.json")))
    m = oracle.OracleModel.from_xml(os.path.join(golden, "gap_water", "GAP.xml"))
    es = []
    for c in d["cell_sizes"]:
        r = m.calc(np.array(d["positions"]), [1, 1], np.eye(3) * c, [1, 1, 1])
        es.append(r["energy"])
    assert np.abs(np.array(es) - np.array(d["ref_energies"])).max() < d["tol"]


def test_oracle_forces_are_energy_gradient(golden):
    """Finite differences of E reproduce F and the virial (pot_test_gradient analogue,
    src/Potentials/Potential.f95:1374-1444)."""
    frames = read_xyz(os.path.join(golden, "Si.np1.xyz"))
    fr = frames[4]  # 16-atom periodic Si cell
    ref = np.load(os.path.join(golden, "si_soap_cur_points.npz"))
    X = ref["sparsex"]
    rng = np.random.default_rng(0)
    parsed = dict(e0={14: -0.5}, coords=[dict(desc_str=SI_SOAP, desc=oracle.parse_args(SI_SOAP), cov=2, delta=3.0, zeta=4.0,
                                              theta=None, M=100, D=325, X=X, alpha=rng.normal(0, 1, 100), sc=np.ones(100))])
    m = oracle.OracleModel(parsed)
    r = m.calc(fr.positions, fr.numbers, fr.lattice)
    h = 1e-5
    for a, k in [(0, 0), (3, 1), (7, 2)]:
        p1 = fr.positions.copy(); p1[a, k] += h
        p2 = fr.positions.copy(); p2[a, k] -= h
        fd = -(m.calc(p1, fr.numbers, fr.lattice)["energy"] - m.calc(p2, fr.numbers, fr.lattice)["energy"]) / (2 * h)
        assert abs(fd - r["force"][a, k]) < 1e-6
    # virial = -dE/d(strain) for a homogeneous deformation
    for a, b in [(0, 0), (0, 1), (2, 1)]:
        eps = np.zeros((3, 3)); eps[a, b] = h
        e1 = m.calc(fr.positions @ (np.eye(3) + eps).T, fr.numbers, (np.eye(3) + eps) @ fr.lattice)["energy"]
        e2 = m.calc(fr.positions @ (np.eye(3) - eps).T, fr.numbers, (np.eye(3) - eps) @ fr.lattice)["energy"]
        assert abs(-(e1 - e2) / (2 * h) - r["virial"][a, b]) < 1e-5
    np.testing.assert_allclose(r["local_virial"].sum(0), r["virial"], atol=1e-10)
    np.testing.assert_allclose(r["local_energy"].sum(), r["energy"], atol=1e-10)


def _random_rotation(seed):
    q, r = np.linalg.qr(np.random.default_rng(seed).normal(size=(3, 3)))
    q = q * np.sign(np.diag(r))
    return q if np.linalg.det(q) > 0 else -q


@pytest.mark.parametrize("case", ["si_fixture", "two_species"])
def test_oracle_rotation_covariance(golden, tmp_path, case):
    """Rotating the atoms with their cell leaves E unchanged and rotates F (F R^T) and
    the virial (R V R^T): checks the real spherical harmonics, the power spectrum and
    the force/virial assembly as a whole, for one and for two species channels."""
    if case == "si_fixture":
        fr = read_xyz(os.path.join(golden, "Si.np1.xyz"))[4]
        X = np.load(os.path.join(golden, "si_soap_cur_points.npz"))["sparsex"]
        parsed = dict(e0={14: -0.5}, coords=[dict(desc_str=SI_SOAP, desc=oracle.parse_args(SI_SOAP), cov=2, delta=3.0,
                                                  zeta=4.0, theta=None, M=100, D=325, X=X,
                                                  alpha=np.random.default_rng(0).normal(0, 1, 100), sc=np.ones(100))])
        m = oracle.OracleModel(parsed)
        pos, Z, lat = fr.positions, fr.numbers, fr.lattice
    else:
        from helpers import sic_model
        m = oracle.OracleModel.from_xml(sic_model(tmp_path))
        at = models.random_triclinic(60, rng=np.random.default_rng(3))
        pos, Z, lat = at.positions, at.numbers, at.lattice
    R = _random_rotation(7)
    r0 = m.calc(pos, Z, lat)
    r1 = m.calc(pos @ R.T, Z, R @ lat)
    n = len(Z)
    assert abs(r1["energy"] - r0["energy"]) < 1e-10 * n
    np.testing.assert_allclose(r1["force"], r0["force"] @ R.T, atol=1e-9)
    np.testing.assert_allclose(r1["virial"], R @ r0["virial"] @ R.T, atol=1e-8)
    np.testing.assert_allclose(r1["local_energy"], r0["local_energy"], atol=1e-10)


def test_oracle_permutation_and_cutoff_continuity(tmp_path):
    """Relabelling the atoms permutes F and local energies and leaves E unchanged; a
    neighbour crossing the SOAP cutoff changes E and F continuously (the cosine
    transition brings fc and fc' to zero at r_c)."""
    from helpers import sic_model
    m = oracle.OracleModel.from_xml(sic_model(tmp_path))
    at = models.random_triclinic(48, rng=np.random.default_rng(5))
    perm = np.random.default_rng(6).permutation(len(at))
    r0 = m.calc(at.positions, at.numbers, at.lattice)
    r1 = m.calc(at.positions[perm], at.numbers[perm], at.lattice)
    assert abs(r1["energy"] - r0["energy"]) < 1e-10 * len(at)
    np.testing.assert_allclose(r1["force"], r0["force"][perm], atol=1e-10)
    np.testing.assert_allclose(r1["local_energy"], r0["local_energy"][perm], atol=1e-10)
    # Si-C dimer in a large cluster box, across the largest cutoff of the model's coordinates
    rc = m.cutoff()
    box = np.eye(3) * 40.0

    def dimer(r):
        return m.calc(np.array([[10.0, 10.0, 10.0], [10.0 + r, 10.0, 10.0]]), np.array([14, 6]), box, [0, 0, 0])

    lo, hi = dimer(rc - 1e-7), dimer(rc + 1e-7)
    assert abs(lo["energy"] - hi["energy"]) < 1e-9
    assert np.abs(lo["force"] - hi["force"]).max() < 1e-6
    assert np.abs(hi["force"]).max() == 0.0       # beyond every cutoff: no interaction


def test_oracle_coordinate_options(golden):
    """only_descriptor and energy_per_coordinate (IPModel_GAP.f95:399-403, :462, :570) on the
    water model's distance_2b coordinates: the per-coordinate energies and the isolated-atom
    energies make up E; selecting one coordinate leaves its energy and its forces only,
    and the selections add up to the full forces."""
    at = _water()
    m = oracle.OracleModel.from_xml(os.path.join(golden, "gap_water", "GAP.xml"))
    args = (at.positions, at.numbers, at.lattice, [1, 1, 1])
    full = m.calc(*args)
    epc = full["energy_per_coordinate"]
    nc = len(epc)
    e0 = full["energy"] - epc.sum()
    f_sum = np.zeros_like(full["force"])
    for k in range(1, nc + 1):
        r = m.calc(*args, only_descriptor=k)
        assert abs(r["energy"] - (e0 + epc[k - 1])) < 1e-9
        np.testing.assert_allclose(r["energy_per_coordinate"], np.where(np.arange(nc) == k - 1, epc, 0.0), atol=1e-12)
        f_sum += r["force"]
    np.testing.assert_allclose(f_sum, full["force"], atol=1e-9)
    if nc > 1:  # a value matching no coordinate evaluates none (the reference's loop skips them all)
        assert abs(m.calc(*args, only_descriptor=0)["energy"] - e0) < 1e-12
