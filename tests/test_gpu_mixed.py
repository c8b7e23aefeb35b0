"""Mixed-precision path (FP32 SOAP, tcgen05 split-BF16 or TF32 kernel GEMMs) against
the FP64 path: force error <= 1 meV/A is the acceptance bound of the mixed form."""
import numpy as np
import pytest

from quip_gb300 import models

from helpers import si_model, sic_model

pytestmark = pytest.mark.gpu

F_TOL_MIXED = 1e-3      # eV/A
E_TOL_MIXED = 1e-4      # eV/atom


def _pair(path, prec):
    from quip_gb300.potential import Potential
    return Potential(param_filename=path, precision="fp64"), Potential(param_filename=path, precision=prec)


@pytest.fixture(scope="module")
def si_gap(tmp_path_factory):
    return si_model(tmp_path_factory.mktemp("si_mixed"))


@pytest.mark.parametrize("prec", ["bf16x3", "tf32", "fp16"])
def test_mixed_si64_vs_fp64(si_gap, prec):
    p64, pm = _pair(si_gap, prec)
    at = models.si_diamond(2, rattle=0.05, seed=7)
    a = p64.calc(at, local_energy=True)
    b = pm.calc(at, local_energy=True)
    de = abs(a["energy"] - b["energy"]) / len(at)
    dle = np.abs(a["local_energy"] - b["local_energy"]).max()
    df = np.abs(a["force"] - b["force"]).max()
    dv = np.abs(a["virial"] - b["virial"]).max()
    print("%s: dE/atom=%.3e dlocalE=%.3e dF=%.3e dV=%.3e |F|max=%.3e" % (prec, de, dle, df, dv, np.abs(a["force"]).max()))
    assert dle < E_TOL_MIXED
    assert de < E_TOL_MIXED
    assert df < F_TOL_MIXED
    assert dv < 1e-2


@pytest.mark.parametrize("prec", ["bf16x3", "tf32", "fp16"])
def test_mixed_two_species_vs_fp64(tmp_path, prec):
    p = sic_model(tmp_path)
    p64, pm = _pair(p, prec)
    at = models.random_triclinic(300, rng=np.random.default_rng(12))
    a, b = p64.calc(at), pm.calc(at)
    df = np.abs(a["force"] - b["force"]).max()
    assert abs(a["energy"] - b["energy"]) / len(at) < E_TOL_MIXED
    assert df < F_TOL_MIXED


def test_mixed_descriptors_close_to_fp64(si_gap):
    p64, pm = _pair(si_gap, "bf16x3")
    at = models.si_diamond(2, rattle=0.05, seed=7)
    q64, q32 = p64.descriptors(at), pm.descriptors(at)
    assert np.abs(q64 - q32).max() < 1e-5


def test_mixed_bitwise_reproducible(si_gap):
    _, pm = _pair(si_gap, "bf16x3")
    at = models.si_diamond(2, rattle=0.05, seed=7)
    r1, r2 = pm.calc(at), pm.calc(at)
    assert r1["energy"] == r2["energy"] and np.array_equal(r1["force"], r2["force"])
