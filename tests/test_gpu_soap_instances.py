"""The fixed-size FP32 SOAP kernels at every basis they are compiled for, against the
generic kernels on the same structure.

Basis sizes select the kernels (L = l_max + 1; NMP = n_max rounded up to a multiple of 4):
the forward with the basis size fixed at compile time (L x NMP = 9x12, 7x8, 5x8, 5x4), the
backward's per-lm h kernel (L, n_max, species = 9,10,2 / 7,8,1 / 5,4,2; the generic h
kernel otherwise) and its thread-per-pair kernel (9x12, 7x8, 5x8, 5x4).  Context options
soap_fwd 0 and soap_bwd 0 select the generic forward and the block-per-centre backward.
The 9x12 instances run at the headline basis (test_gpu_headline_parity.py); here:

* at each other instance basis the two paths sum in different orders, so their results
  differ in the last bits (which shows that the fixed-size kernel ran) and agree to
  energy 1e-8 eV/atom, forces 1e-6 eV/A, virial 1e-5 eV (measured on a GB300: at most
  1.6e-12 eV/atom, 7.2e-9 eV/A and 1.8e-7 eV); the backward leaves the energy unchanged;
* at a basis with no instance the options change nothing: bit-identical results.
"""
import os

import numpy as np
import pytest

from quip_gb300 import models

from helpers import oracle_descriptor_fn

pytestmark = pytest.mark.gpu

# (n_max, l_max, species, compiled instance)
BASES = {
    "5x4-two-species": (4, 4, (14, 6), True),     # forward 5x4, h 5,4,2, pairs 5x4
    "7x8-one-species": (8, 6, (14,), True),       # forward 7x8, h 7,8,1, pairs 7x8
    "5x8-generic-h": (5, 4, (14,), True),         # forward 5x8, generic h, pairs 5x8
    "6x8-no-instance": (6, 5, (14,), False),      # generic forward, block backward
}


def _model(tmp_path, n_max, l_max, species):
    if len(species) == 1:
        structs = [models.si_diamond(2, rattle=0.05 + 0.05 * k, seed=200 + k) for k in range(2)]
    else:
        structs = [models.random_binary(96, seed=400 + k) for k in range(2)]
    path = os.path.join(str(tmp_path), "gap_%d_%d_%d.xml" % (n_max, l_max, len(species)))
    return models.random_soap_gap(path, oracle_descriptor_fn, structs, n_max=n_max, l_max=l_max, cutoff=4.5,
                                  width=1.0, atom_sigma=0.5, species=species, M=100, zeta=4.0, delta=1.0,
                                  with_2b=False, seed=7)


def _cell(species):
    if len(species) == 1:
        return models.si_diamond(3, rattle=0.1, seed=9)
    return models.random_binary(160, seed=11)


def _pot(path, **options):
    from quip_gb300.potential import Potential
    p = Potential(param_filename=path, precision="tf32")
    for k, v in options.items():
        p.set_option(k, v)
    return p


@pytest.mark.parametrize("basis", sorted(BASES))
def test_fixed_forward_against_generic(tmp_path, basis):
    n_max, l_max, species, instance = BASES[basis]
    path = _model(tmp_path, n_max, l_max, species)
    at = _cell(species)
    ra = _pot(path).calc(at)
    rb = _pot(path, soap_fwd=0).calc(at)
    de = abs(ra["energy"] - rb["energy"]) / len(at)
    df = np.abs(ra["force"] - rb["force"]).max()
    dv = np.abs(ra["virial"] - rb["virial"]).max()
    print("%s: fixed-size vs generic forward: dE/atom=%.2e dF=%.2e dV=%.2e" % (basis, de, df, dv))
    if instance:
        assert not np.array_equal(ra["force"], rb["force"])
        assert de < 1e-8 and df < 1e-6 and dv < 1e-5
    else:
        assert ra["energy"] == rb["energy"]
        assert np.array_equal(ra["force"], rb["force"]) and np.array_equal(ra["virial"], rb["virial"])


@pytest.mark.parametrize("basis", sorted(BASES))
def test_pair_backward_against_block(tmp_path, basis):
    n_max, l_max, species, instance = BASES[basis]
    path = _model(tmp_path, n_max, l_max, species)
    at = _cell(species)
    ra = _pot(path).calc(at)
    rb = _pot(path, soap_bwd=0).calc(at)
    df = np.abs(ra["force"] - rb["force"]).max()
    dv = np.abs(ra["virial"] - rb["virial"]).max()
    print("%s: thread-per-pair vs block backward: dF=%.2e dV=%.2e" % (basis, df, dv))
    assert ra["energy"] == rb["energy"]
    if instance:
        assert not np.array_equal(ra["force"], rb["force"])
        assert df < 1e-6 and dv < 1e-5
    else:
        assert np.array_equal(ra["force"], rb["force"]) and np.array_equal(ra["virial"], rb["virial"])
