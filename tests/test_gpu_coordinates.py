"""Calc arguments that act per GP coordinate (IPModel_GAP.f95:334-335, :399-403, :462, :570):
only_descriptor=<k> evaluates only coordinate k (1-based) of a model with more than one;
energy_per_coordinate=<name> returns, per coordinate, the sum of e_i * covariance_cutoff
over the evaluated descriptor instances (before E_scale, without e0).  Against the oracle,
which restates the same loop; the SiC model has one SOAP and three distance_2b coordinates.
"""
import numpy as np
import pytest

from oracle import oracle
from quip_gb300 import _lib, models

from helpers import si_model, sic_model

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sic_gap(tmp_path_factory):
    return sic_model(tmp_path_factory.mktemp("sic_coords"))


def _pot(path, precision="fp64"):
    from quip_gb300.potential import Potential
    return Potential(param_filename=path, precision=precision)


def _structure(n=90, seed=11):
    return models.random_triclinic(n, rng=np.random.default_rng(seed))


@pytest.mark.parametrize("masked", [False, True])
def test_energy_per_coordinate_vs_oracle(sic_gap, masked):
    pot, om = _pot(sic_gap), oracle.OracleModel.from_xml(sic_gap)
    at = _structure()
    mask = (np.arange(len(at)) % 3 != 1).astype(np.int32) if masked else None
    r = pot.calc(at, atom_mask=mask, args_str="energy_per_coordinate=epc")
    o = om.calc(at.positions, at.numbers, at.lattice, at.pbc.astype(int), mask=mask)
    assert r["epc"].shape == (4,)
    assert np.abs(r["epc"] - o["energy_per_coordinate"]).max() < 1e-9 * len(at)
    # the coordinates' shares and the isolated-atom energies make up the energy
    e0 = o["energy"] - o["energy_per_coordinate"].sum()
    assert abs(r["epc"].sum() + e0 - r["energy"]) < 1e-9 * len(at)


def test_energy_per_coordinate_tf32(sic_gap):
    pot, om = _pot(sic_gap, "tf32"), oracle.OracleModel.from_xml(sic_gap)
    at = _structure(140, 12)
    r = pot.calc(at, args_str="energy_per_coordinate=epc")
    o = om.calc(at.positions, at.numbers, at.lattice, at.pbc.astype(int))
    assert np.abs(r["epc"] - o["energy_per_coordinate"]).max() < 1e-5 * len(at)


@pytest.mark.parametrize("k", [1, 2, 4])
def test_only_descriptor_vs_oracle(sic_gap, k):
    pot, om = _pot(sic_gap), oracle.OracleModel.from_xml(sic_gap)
    at = _structure(70, 13)
    r = pot.calc(at, local_energy=True, args_str="only_descriptor=%d energy_per_coordinate=epc" % k)
    o = om.calc(at.positions, at.numbers, at.lattice, at.pbc.astype(int), only_descriptor=k)
    n = len(at)
    assert abs(r["energy"] - o["energy"]) / n < 1e-8
    assert np.abs(r["force"] - o["force"]).max() < 1e-7
    assert np.abs(r["virial"] - o["virial"]).max() < 1e-7
    assert np.abs(r["local_energy"] - o["local_energy"]).max() < 1e-7
    assert np.abs(r["epc"] - o["energy_per_coordinate"]).max() < 1e-9 * n
    assert np.count_nonzero(r["epc"]) == 1 and r["epc"][k - 1] != 0.0


def test_only_descriptor_single_coordinate_model_evaluates_it(tmp_path):
    path = si_model(tmp_path, M=120, with_2b=False)
    pot = _pot(path)
    at = models.si_diamond(2, rattle=0.05, seed=3)
    full = pot.calc(at)
    assert len(pot.info()) == 1
    sel = pot.calc(at, args_str="only_descriptor=5")     # ignored with one coordinate (:399)
    assert sel["energy"] == full["energy"] and np.array_equal(sel["force"], full["force"])


def test_energy_per_coordinate_in_batches_and_graphs(sic_gap):
    pot = _pot(sic_gap, "tf32")
    rng = np.random.default_rng(14)
    structs = [models.random_triclinic(int(k), rng=rng) for k in (30, 75, 52)]
    batch = pot.calc_batch(structs, args_str="energy_per_coordinate=epc")
    for at, b in zip(structs, batch):
        a = pot.calc(at, args_str="energy_per_coordinate=epc")
        assert np.array_equal(a["epc"], b["epc"])
    pot.set_option("graphs", 1)
    at = structs[1]
    ref = pot.calc(at, args_str="energy_per_coordinate=epc")["epc"]
    for _ in range(3):
        assert np.array_equal(pot.calc(at, args_str="energy_per_coordinate=epc")["epc"], ref)
    # a plain call in between: the sums are not requested, and asking for them fails
    pot.calc(at)
    out = np.zeros(4)
    cnt = _lib.ctypes.c_int()
    rc = pot._L.gapgpu_energy_per_coordinate(pot._ctx, _lib.ptr(out), 4, _lib.ctypes.byref(cnt))
    assert rc == _lib.ERR_ARG
    assert np.array_equal(pot.calc(at, args_str="energy_per_coordinate=epc")["epc"], ref)
