"""The oracle's GAP variance estimate (local_gap_variance / gap_variance_gradient,
IPModel_GAP.f95:464-488) on its own, without a GPU.

No reference fixture pins the variance (its estimator lives in the absent GAP
submodule), so the restatement is held to the properties it must have:
* sigma^2 = k(x,x) - k^T (K_MM + lambda I)^-1 k is non-negative, and at a sparse point it
  is of the order of the regularisation lambda;
* gap_variance_gradient(:, j) is the derivative of sum_a local_gap_variance(a) with
  respect to r_j (central differences, SOAP and distance_2b coordinates together).
"""
import numpy as np
import pytest

from oracle import oracle
from quip_gb300 import models

from helpers import oracle_descriptor_fn


@pytest.fixture(scope="module")
def small_model(tmp_path_factory):
    d = tmp_path_factory.mktemp("var")
    structs = [models.si_diamond(1, rattle=0.1, seed=30 + k) for k in range(8)]
    return models.random_soap_gap(str(d / "var_gap.xml"), oracle_descriptor_fn, structs, n_max=4, l_max=3, cutoff=4.0,
                                  width=1.0, atom_sigma=0.5, species=(14,), M=40, zeta=2.0, delta=1.0, seed=4,
                                  with_2b=True, M2=10)


def _om(path, reg=1e-3):
    om = oracle.OracleModel.from_xml(path)
    om.init_variance(reg)
    return om


def test_variance_is_nonnegative_and_small_at_a_sparse_point(small_model):
    om = _om(small_model)
    at = models.si_diamond(1, rattle=0.1, seed=30)   # one of the structures the sparse points came from
    v = om.variance(at.positions, at.numbers, at.lattice, gradient=False)
    assert np.all(v["instance_variance"] > -1e-12)
    assert np.all(v["local_gap_variance"] > -1e-12)
    # some SOAP instance of this structure is a sparse point: its variance is ~ lambda
    assert v["instance_variance"][:len(at)].min() < 1e-2


def test_variance_gradient_is_the_derivative_of_the_summed_local_variance(small_model):
    om = _om(small_model)
    at = models.si_diamond(1, rattle=0.15, seed=77)
    v = om.variance(at.positions, at.numbers, at.lattice)
    h = 1e-5
    for a in (0, 3, 6):
        for k in range(3):
            p = at.positions.copy()
            p[a, k] += h
            up = om.variance(p, at.numbers, at.lattice, gradient=False)["local_gap_variance"].sum()
            p[a, k] -= 2 * h
            dn = om.variance(p, at.numbers, at.lattice, gradient=False)["local_gap_variance"].sum()
            fd = (up - dn) / (2 * h)
            assert abs(fd - v["gap_variance_gradient"][a, k]) < 1e-6 * max(1.0, abs(fd)), (a, k, fd)


def test_variance_needs_the_set_up(small_model):
    om = oracle.OracleModel.from_xml(small_model)
    at = models.si_diamond(1, rattle=0.1, seed=3)
    with pytest.raises(RuntimeError):
        om.variance(at.positions, at.numbers, at.lattice)
