"""Sparse-GP GEMMs on CTA pairs (tcgen05 cta_group::2, 256-row tiles) against the
single-CTA tiles: same energies, forces and virials to TF32 round-off, with row counts
that leave partial and empty halves of the last 256-row tile."""
import numpy as np
import pytest

from quip_gb300 import models

from helpers import oracle_descriptor_fn, sic_model

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sic_gap(tmp_path_factory):
    return sic_model(tmp_path_factory.mktemp("sic_pairs"))


@pytest.fixture(scope="module")
def sic_gap_tails(tmp_path_factory):
    # D = 276 and M = 300 pad to 384: both GEMMs end in a 128-wide tile after a 256-wide one
    rng = np.random.default_rng(3)
    structs = [models.random_triclinic(int(n), rng=rng) for n in (40, 48, 56, 64, 40, 48, 56, 64)]
    path = str(tmp_path_factory.mktemp("sic_pairs_tail") / "sic_gap.xml")
    return models.random_soap_gap(path, oracle_descriptor_fn, structs, n_max=5, l_max=4, cutoff=4.5, width=1.0,
                                  atom_sigma=0.5, species=(14, 6), M=300, zeta=4.0, delta=1.0, with_2b=True, seed=3)


def _pot(path, pairs, f16=0):
    from quip_gb300.potential import Potential
    pot = Potential(param_filename=path, precision="tf32")
    pot.set_option("pairs", pairs)
    pot.set_option("gemm2_f16", f16)  # tile tests: TF32 GEMMs on both sides
    pot.set_option("gemm1_f16", f16)
    return pot


@pytest.mark.parametrize("n,tails", [(37, False), (300, False), (520, False), (300, True)])
def test_pair_tiles_match_single_cta_tiles(sic_gap, sic_gap_tails, n, tails):
    path = sic_gap_tails if tails else sic_gap
    at = models.random_triclinic(n, rng=np.random.default_rng(100 + n))
    ref = _pot(path, 0).calc(at, local_energy=True)
    got = _pot(path, 2).calc(at, local_energy=True)
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


@pytest.mark.parametrize("g1,g2", [(0, 1), (1, 1), (1, 0)])
@pytest.mark.parametrize("n", [37, 300])
def test_fp16_gemms_match_tf32(sic_gap, n, g1, g2):
    """The sparse-GP GEMMs in FP16 on CTA pairs -- K = Q X^T (FP16 descriptors and sparse
    points) and/or G = W X (W' = S K^(zeta-1), X' = coef zeta / S x) -- against the TF32
    GEMMs and against FP64 (FP16 and TF32 both carry 10-bit mantissas)."""
    from quip_gb300.potential import Potential
    at = models.random_triclinic(n, rng=np.random.default_rng(200 + n))
    ref = _pot(sic_gap, 1, f16=0)
    ref.set_option("gemm1_f16", 0)
    ref = ref.calc(at)
    pot = _pot(sic_gap, 1, f16=g2)
    pot.set_option("gemm1_f16", g1)
    got = pot.calc(at)
    exact = Potential(param_filename=sic_gap, precision="fp64").calc(at)
    scale = max(1.0, np.abs(exact["force"]).max())
    for r in (ref, got):
        assert abs(r["energy"] - exact["energy"]) <= 1e-5 * n
        assert np.abs(r["force"] - exact["force"]).max() <= 1e-4 * scale
    assert np.abs(got["force"] - ref["force"]).max() <= 1e-4 * scale
    if not g1:  # energies come from the first GEMM
        assert got["energy"] == pytest.approx(ref["energy"], abs=1e-9 * n)
