"""Shared fixtures for the parity tests: seeded structures and random GAP models whose
sparse points are SOAP vectors computed by the oracle."""
import os

import numpy as np

from oracle import oracle
from quip_gb300 import models


def oracle_descriptor_fn(desc, at):
    return oracle.soap(desc, at.positions, at.numbers, at.lattice, at.pbc)


def si_model(tmp, n_max=8, l_max=6, M=500, seed=0, with_2b=True, zeta=4.0):
    """The 64-atom benchmark model family: SOAP n_max=8 l_max=6 rc=5 (D=253), M sparse
    points from seeded rattled diamond cells, alpha ~ N(0, 1e-3), plus distance_2b."""
    structs = [models.si_diamond(2, rattle=0.05 + 0.05 * k, seed=100 + k) for k in range(max(1, M // 64 + 1))]
    path = os.path.join(str(tmp), "si_gap.xml")
    return models.random_soap_gap(path, oracle_descriptor_fn, structs, n_max=n_max, l_max=l_max, cutoff=5.0, width=1.0,
                                  atom_sigma=0.5, species=(14,), M=M, zeta=zeta, delta=1.0, with_2b=with_2b, seed=seed)


def sic_model(tmp, n_max=4, l_max=4, M=200, seed=1):
    rng = np.random.default_rng(seed)
    structs = [models.random_triclinic(int(n), rng=rng) for n in (24, 40, 64, 80)]
    path = os.path.join(str(tmp), "sic_gap.xml")
    return models.random_soap_gap(path, oracle_descriptor_fn, structs, n_max=n_max, l_max=l_max, cutoff=4.5, width=1.0,
                                  atom_sigma=0.5, species=(14, 6), M=M, zeta=4.0, delta=1.0, with_2b=True, seed=seed)
