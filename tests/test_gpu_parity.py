"""GPU (libgapgpu, sm_103a) against the FP64 oracle and the reference fixtures.

Plain FP64 path tolerances (stated by the benchmark contract): energy <= 1e-8 eV/atom,
forces <= 1e-7 eV/A.  Virials are held to 1e-7 eV per component.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle
from quip_gb300 import models
from quip_gb300.atoms import read_xyz

from helpers import si_model, sic_model

pytestmark = pytest.mark.gpu

E_TOL_PER_ATOM = 1e-8
F_TOL = 1e-7
V_TOL = 1e-7


def _pot(path, precision="fp64"):
    from quip_gb300.potential import Potential
    return Potential(param_filename=path, precision=precision)


def _compare(pot, om, at, mask=None, e_tol=E_TOL_PER_ATOM, f_tol=F_TOL, v_tol=V_TOL):
    r = pot.calc(at, local_energy=True, local_virial=True, atom_mask=mask)
    o = om.calc(at.positions, at.numbers, at.lattice, at.pbc.astype(int), mask=mask)
    n = len(at)
    assert abs(r["energy"] - o["energy"]) / n < e_tol, (r["energy"], o["energy"])
    assert np.abs(r["force"] - o["force"]).max() < f_tol
    assert np.abs(r["virial"] - o["virial"]).max() < v_tol
    assert np.abs(r["local_energy"] - o["local_energy"]).max() < e_tol * 10
    assert np.abs(r["local_virial"] - o["local_virial"]).max() < v_tol
    return r, o


def test_water_distance_2b_fixture(golden):
    at = read_xyz(os.path.join(golden, "gap_water", "gap_sample.xyz"))[0]
    path = os.path.join(golden, "gap_water", "GAP.xml")
    pot = _pot(path)
    r = pot.calc(at)
    assert abs(r["energy"] - at.info["energy"]) < 1e-5          # tests/test_gappot.py:45
    assert np.abs(r["force"] - at.arrays["force"]).max() < 1e-6  # tests/test_gappot.py:48
    om = oracle.OracleModel.from_xml(path)
    # the alphas are ~1e6, so agreement is limited by cancellation, not by the method
    _compare(pot, om, at, e_tol=1e-9, f_tol=1e-7, v_tol=1e-6)


def test_potential_cell_energies(golden):
    d = json.load(open(os.path.join(golden, "potential_cell.json")))
    pot = _pot(os.path.join(golden, "gap_water", "GAP.xml"))
    es = []
    for c in d["cell_sizes"]:
        at = models.Atoms([1, 1], np.array(d["positions"]), lattice=np.eye(3) * c, pbc=True)
        es.append(pot.calc(at, force=False, virial=False)["energy"])
    assert np.abs(np.array(es) - np.array(d["ref_energies"])).max() < d["tol"]


def test_soap_descriptors_match_reference_vectors(golden, tmp_path):
    ref = np.load(os.path.join(golden, "si_soap_cur_points.npz"))
    X, idx = ref["sparsex"], ref["index"]
    desc = ("soap atom_sigma=0.5 central_weight=1.0 cutoff=4.0 cutoff_transition_width=1.0 l_max=8 n_max=8 "
            "n_species=1 species_Z={14} Z=14")
    p = models.write_gap_xml(str(tmp_path / "si_fix.xml"), [dict(desc_str=desc, cov="dot_product", delta=3.0, zeta=4.0,
                                                                X=X, alpha=ref["alpha"], sc=np.ones(len(X)))])
    pot = _pot(p)
    frames = read_xyz(os.path.join(golden, "Si.np1.xyz"))
    where = [(f, k) for f, fr in enumerate(frames) for k in range(len(fr))]
    worst = 0.0
    cache = {}
    for t, gi in enumerate(idx):
        f, k = where[gi - 1]
        if f not in cache:
            cache[f] = pot.descriptors(frames[f], 0)
        worst = max(worst, np.abs(cache[f][k] - X[t]).max())
    assert worst < 1e-8, worst


@pytest.fixture(scope="module")
def si_gap(tmp_path_factory):
    return si_model(tmp_path_factory.mktemp("si"))


def test_si64_soap_gap_vs_oracle(si_gap):
    pot, om = _pot(si_gap), oracle.OracleModel.from_xml(si_gap)
    at = models.si_diamond(2, rattle=0.05, seed=7)
    _compare(pot, om, at)


def test_si_primitive_periodic_images(si_gap):
    """2-atom cell, cutoff 5 A > cell width 3.13 A: every image is a separate neighbour."""
    pot, om = _pot(si_gap), oracle.OracleModel.from_xml(si_gap)
    at = models.si_primitive(rattle=0.03, seed=3)
    _compare(pot, om, at)


def test_si4096_soap_gap_vs_oracle(tmp_path):
    p = si_model(tmp_path, M=2000, seed=5)
    pot, om = _pot(p), oracle.OracleModel.from_xml(p)
    at = models.si_diamond(8, rattle=0.1, seed=11)
    _compare(pot, om, at)


def test_two_species_soap_vs_oracle(tmp_path):
    p = sic_model(tmp_path)
    pot, om = _pot(p), oracle.OracleModel.from_xml(p)
    at = models.random_triclinic(60, rng=np.random.default_rng(9))
    _compare(pot, om, at)


def test_atom_mask_vs_oracle(si_gap):
    pot, om = _pot(si_gap), oracle.OracleModel.from_xml(si_gap)
    at = models.si_diamond(2, rattle=0.05, seed=8)
    mask = (np.arange(len(at)) % 3 == 0).astype(np.int32)
    _compare(pot, om, at, mask=mask)


def test_neighbour_list_matches_oracle(si_gap):
    pot = _pot(si_gap)
    rng = np.random.default_rng(4)
    cases = [models.si_diamond(2, rattle=0.05, seed=1), models.si_primitive(rattle=0.02),
             models.random_triclinic(50, rng=rng), models.random_triclinic(9, rng=rng)]
    cl = models.si_diamond(2, rattle=0.05, seed=2)
    cl.pbc = np.array([False, False, False])
    cases.append(cl)
    mixed = models.si_diamond(2, rattle=0.05, seed=3)
    mixed.pbc = np.array([True, False, True])
    cases.append(mixed)
    for at in cases:
        off, j, sh = pot.neighbours(at, 5.0)
        o_off, o_j, o_sh, _, _ = oracle.neighbours(at.positions, at.lattice, at.pbc.astype(int), 5.0)
        np.testing.assert_array_equal(np.diff(off), np.diff(o_off))
        for a in range(len(at)):
            g = sorted((int(j[p]),) + tuple(sh[p]) for p in range(off[a], off[a + 1]))
            o = sorted((int(o_j[p]),) + tuple(o_sh[p]) for p in range(o_off[a], o_off[a + 1]))
            assert g == o


def _cubic_grid(n=4, a=2.5):
    g = np.stack(np.meshgrid(range(n), range(n), range(n), indexing="ij"), -1).reshape(-1, 3) * a
    return models.Atoms(np.full(len(g), 14), g, lattice=np.eye(3) * (n * a))


def _faces_and_outside():
    """Atoms on cell faces (fractional 0.5, -0.5, 1.0), at the largest double below 0.5,
    and several cells outside the cell, where the wrap map_shift = -floor(s + 0.5)
    (Connection.f95:1573-1579) decides the shifts."""
    frac = np.array([[0.5, 0.5, 0.5], [-0.5, 0.0, 0.25], [1.0, 1.0, 0.5], [0.0, 0.0, 0.0],
                     [3.7, -2.2, np.nextafter(0.5, 0.0)], [0.5, -0.5, 1.25], [-1.0, 2.0, -2.75],
                     [0.25, 0.75, 0.125]])
    lat = np.array([[6.0, 0.0, 0.0], [1.5, 5.5, 0.0], [-1.0, 0.75, 7.0]]).T
    return models.Atoms(np.full(len(frac), 14), frac @ lat.T, lattice=lat)


def _same_lists(got, ref, n):
    off, j, sh = got
    o_off, o_j, o_sh = ref[:3]
    np.testing.assert_array_equal(np.diff(off), np.diff(o_off))
    for a in range(n):
        g = sorted((int(j[p]),) + tuple(sh[p]) for p in range(off[a], off[a + 1]))
        o = sorted((int(o_j[p]),) + tuple(o_sh[p]) for p in range(o_off[a], o_off[a + 1]))
        assert g == o


@pytest.mark.parametrize("precision", ["fp64", "tf32"])
def test_neighbour_list_edges(si_gap, precision):
    """Pairs exactly at the cutoff are out (strict <, Connection.f95:517) and the next
    double above brings them in: on a 2.5 A cubic grid the shells at 2.5, 3.54 and 4.33 A
    give 26 neighbours below 5.0 A and the 5.0 A shell 6 more.  The FP32 pre-test of the
    mixed build leaves these exact-distance pairs to the FP64 test, so both precisions
    give the same lists."""
    pot = _pot(si_gap, precision)
    grid = _cubic_grid()
    for rc, count in ((5.0, 26), (np.nextafter(5.0, 0.0), 26), (np.nextafter(5.0, 6.0), 32),
                      (2.5, 0), (np.nextafter(2.5, 3.0), 6)):
        got = pot.neighbours(grid, float(rc))
        assert set(np.diff(got[0]).tolist()) == {count}, rc
        _same_lists(got, oracle.neighbours(grid.positions, grid.lattice, [1, 1, 1], float(rc)), len(grid))
    at = _faces_and_outside()
    for rc in (4.0, 7.5):
        _same_lists(pot.neighbours(at, rc), oracle.neighbours(at.positions, at.lattice, [1, 1, 1], rc), len(at))


def test_faces_and_outside_vs_oracle(si_gap):
    _compare(_pot(si_gap), oracle.OracleModel.from_xml(si_gap), _faces_and_outside())


def test_bitwise_reproducible(si_gap):
    pot = _pot(si_gap)
    at = models.si_diamond(2, rattle=0.05, seed=7)
    r1 = pot.calc(at)
    r2 = pot.calc(at)
    assert r1["energy"] == r2["energy"]
    assert np.array_equal(r1["force"], r2["force"])
    assert np.array_equal(r1["virial"], r2["virial"])


def test_translation_and_lattice_invariance(si_gap):
    pot = _pot(si_gap)
    at = models.si_diamond(2, rattle=0.05, seed=7)
    e = pot.calc(at)["energy"]
    moved = at.copy()
    moved.positions = moved.positions + np.array([3.1, -7.7, 100.25])
    assert abs(pot.calc(moved)["energy"] - e) < 1e-9 * len(at)
    shifted = at.copy()
    shifted.positions = shifted.positions + at.lattice[:, 0] * 2 - at.lattice[:, 2]
    assert abs(pot.calc(shifted)["energy"] - e) < 1e-9 * len(at)


def test_calc_errors_are_reported(si_gap):
    from quip_gb300._lib import GapGpuError
    pot = _pot(si_gap)
    at = models.si_diamond(2, rattle=0.05, seed=7)
    with pytest.raises(GapGpuError, match="r_scale"):
        pot.calc(at, args_str="r_scale=1.1")
    bad = at.copy()
    bad.positions[1] = bad.positions[0]
    with pytest.raises(GapGpuError, match="overlapping"):
        pot.calc(bad)
    nanat = at.copy()
    nanat.positions[3, 1] = np.nan
    with pytest.raises(GapGpuError, match="NaN"):
        pot.calc(nanat)
    # the context stays usable after an error
    assert np.isfinite(pot.calc(at)["energy"])
