"""Sparse-GP GEMMs on CTA pairs (tcgen05 cta_group::2, 256-row tiles) against the
single-CTA tiles: same energies, forces and virials to TF32 round-off, with row counts
that leave partial and empty halves of the last 256-row tile."""
import numpy as np
import pytest

from quip_gb300 import models

from helpers import sic_model

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sic_gap(tmp_path_factory):
    return sic_model(tmp_path_factory.mktemp("sic_pairs"))


def _pot(path, pairs):
    from quip_gb300.potential import Potential
    pot = Potential(param_filename=path, precision="tf32")
    pot.set_option("pairs", pairs)
    return pot


@pytest.mark.parametrize("n", [37, 300, 520])
def test_pair_tiles_match_single_cta_tiles(sic_gap, n):
    at = models.random_triclinic(n, rng=np.random.default_rng(100 + n))
    ref = _pot(sic_gap, 0).calc(at, local_energy=True)
    got = _pot(sic_gap, 2).calc(at, local_energy=True)
    scale = max(1.0, np.abs(ref["force"]).max())
    assert abs(got["energy"] - ref["energy"]) <= 1e-6 * max(1.0, abs(ref["energy"]))
    assert np.abs(got["force"] - ref["force"]).max() <= 1e-5 * scale
    assert np.abs(got["virial"] - ref["virial"]).max() <= 1e-5 * max(1.0, np.abs(ref["virial"]).max())
    assert np.abs(got["local_energy"] - ref["local_energy"]).max() <= 1e-6 * max(1.0, np.abs(ref["local_energy"]).max())


def test_pair_tiles_in_batches_and_graph_replay(sic_gap):
    pot = _pot(sic_gap, 2)
    rng = np.random.default_rng(7)
    structs = [models.random_triclinic(int(k), rng=rng) for k in (40, 130, 75)]
    batch = pot.calc_batch(structs)
    for at, b in zip(structs, batch):
        a = pot.calc(at)
        assert a["energy"] == b["energy"]
        assert np.array_equal(a["force"], b["force"])
    pot.set_option("graphs", 1)
    at = structs[1]
    ref = pot.calc(at)
    for _ in range(3):
        r = pot.calc(at)
        assert r["energy"] == ref["energy"] and np.array_equal(r["force"], ref["force"])
