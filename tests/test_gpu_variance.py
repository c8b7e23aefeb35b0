"""GAP variance estimate on the GPU (local_gap_variance, gap_variance_gradient,
print_gap_variance; IPModel_GAP.f95:330-335, :464-488, :506-516) against the oracle.

The estimator is set up by the init argument gap_variance_regularisation (:170-187).  No
reference fixture pins it (its arithmetic is in the absent GAP submodule); the oracle's
restatement is checked against finite differences in test_oracle_variance.py, and here the
GPU, which computes the variance in FP64 in every precision, is held to the oracle:
* FP64 context: per-atom variance <= 1e-9, gradient <= 1e-8 (absolute; the values are
  O(1e-2) .. O(1));
* mixed contexts (FP32 descriptors promoted to FP64): per-atom variance within 1e-5 and the
  gradient within 1e-3 of the oracle.
"""
import numpy as np
import pytest

from oracle import oracle
from quip_gb300 import _lib, models

from helpers import sic_model

pytestmark = pytest.mark.gpu

REG = 1e-3


@pytest.fixture(scope="module")
def sic_gap(tmp_path_factory):
    return sic_model(tmp_path_factory.mktemp("sic_var"))


def _pot(path, precision="fp64", variance=True):
    from quip_gb300.potential import Potential
    args = "IP GAP" + (" gap_variance_regularisation=%g" % REG if variance else "")
    return Potential(args_str=args, param_filename=path, precision=precision)


def _oracle(path, at):
    om = oracle.OracleModel.from_xml(path)
    om.init_variance(REG)
    return om.variance(at.positions, at.numbers, at.lattice, at.pbc.astype(int))


@pytest.mark.parametrize("prec", ["fp64", "fp16"])
def test_local_variance_and_gradient_match_oracle(sic_gap, prec):
    at = models.random_triclinic(90, rng=np.random.default_rng(8))
    r = _pot(sic_gap, prec).calc(at, args_str="local_gap_variance=gap_var")
    o = _oracle(sic_gap, at)
    dv = np.abs(r["gap_var"] - o["local_gap_variance"]).max()
    dg = np.abs(r["gap_variance_gradient"] - o["gap_variance_gradient"]).max()
    print("%s: max variance %.3e, d variance %.2e, d gradient %.2e (max |grad| %.3e)"
          % (prec, o["local_gap_variance"].max(), dv, dg, np.abs(o["gap_variance_gradient"]).max()))
    v_tol, g_tol = (1e-9, 1e-8) if prec == "fp64" else (1e-5, 1e-3)
    assert dv < v_tol and dg < g_tol


def test_variance_leaves_energy_and_forces_unchanged(sic_gap):
    at = models.random_triclinic(60, rng=np.random.default_rng(9))
    pot = _pot(sic_gap)
    a = pot.calc(at)
    b = pot.calc(at, args_str="local_gap_variance=v")
    assert a["energy"] == b["energy"] and np.array_equal(a["force"], b["force"])
    assert np.array_equal(a["virial"], b["virial"])


def test_print_gap_variance_lists_every_instance(sic_gap, capsys):
    at = models.random_triclinic(40, rng=np.random.default_rng(10))
    pot = _pot(sic_gap)
    pot.calc(at, args_str="print_gap_variance=T")
    lines = [l for l in capsys.readouterr().out.splitlines() if " var( " in l]
    o = _oracle(sic_gap, at)
    assert len(lines) == len(o["instance_variance"])
    got = np.sort([float(l.split("=")[1].split("*")[0]) for l in lines])
    assert np.abs(got - np.sort(o["instance_variance"])).max() < 1e-9


def test_variance_needs_the_init_argument(sic_gap):
    at = models.random_triclinic(30, rng=np.random.default_rng(11))
    with pytest.raises(_lib.GapGpuError) as e:
        _pot(sic_gap, variance=False).calc(at, args_str="local_gap_variance=v")
    assert e.value.code == _lib.ERR_ARG and "gap_variance_regularisation" in str(e.value)
    with pytest.raises(_lib.GapGpuError) as e:
        _pot(sic_gap).calc_batch([at], args_str="local_gap_variance=v")
    assert e.value.code == _lib.ERR_UNSUPPORTED
