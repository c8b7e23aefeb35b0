"""The LAMMPS pair_style quip path (gapgpu_calc_lammps) against the periodic evaluation.

quip_lammps_wrapper (src/Potentials/quip_lammps_wrapper.f95:30-156) receives explicit
ghost atoms and the host's full neighbour list of each local atom, masks the centres
to the local atoms and returns forces on locals and ghosts.  Built here from a periodic
structure: every periodic image in the neighbour list becomes a ghost; the energy and
virial must equal the periodic calculation's, and local forces and local energies plus
the ghosts' folded back onto their owners must equal the periodic ones.
"""
import numpy as np
import pytest

from oracle import oracle
from quip_gb300 import _lib, models

from helpers import sic_model

pytestmark = pytest.mark.gpu


def _lammps_view(at, cutoff):
    off, j, sh, _, _ = oracle.neighbours(at.positions, at.lattice, at.pbc.astype(int), cutoff)
    n = len(at)
    ghosts, owner = {}, []
    gpos = []
    neigh = []
    for a in range(n):
        for p in range(off[a], off[a + 1]):
            key = (int(j[p]),) + tuple(int(x) for x in sh[p])
            if any(key[1:]):
                if key not in ghosts:
                    ghosts[key] = n + len(owner)
                    owner.append(key[0])
                    gpos.append(at.positions[key[0]] + at.lattice @ np.array(key[1:]))
                neigh.append(ghosts[key] + 1)      # 1-based, as quip_lammps_wrapper reads them
            else:
                neigh.append(key[0] + 1)
    pos = np.concatenate([at.positions, np.array(gpos).reshape(-1, 3)])
    Z = np.concatenate([at.numbers, at.numbers[owner]]).astype(np.int32)
    return pos, Z, np.diff(off).astype(np.int32), np.array(neigh, np.int32), np.array(owner, dtype=int)


@pytest.mark.parametrize("prec", ["fp64", "tf32"])
def test_lammps_path_matches_periodic_calc(tmp_path, prec):
    from quip_gb300.potential import Potential
    path = sic_model(tmp_path)
    pot = Potential(param_filename=path, precision=prec)
    at = models.random_triclinic(70, rng=np.random.default_rng(31))
    ref = pot.calc(at, local_energy=True)
    pos, Z, num, neigh, owner = _lammps_view(at, pot.cutoff())
    n, nloc = len(pos), len(at)
    ilist = np.arange(nloc, dtype=np.int32)
    lat = np.asfortranarray(at.lattice).ravel(order="F").copy()
    E = np.zeros(1)
    F = np.zeros((n, 3))
    V = np.zeros(9)
    LE = np.zeros(n)
    LV = np.zeros((n, 9))
    _lib.check(pot._L.gapgpu_calc_lammps(pot._ctx, nloc, n - nloc, _lib.ptr(Z), nloc, _lib.ptr(ilist), _lib.ptr(num),
                                         _lib.ptr(neigh), _lib.ptr(lat), _lib.ptr(np.ascontiguousarray(pos)),
                                         _lib.ptr(E), _lib.ptr(LE), _lib.ptr(V), _lib.ptr(LV), _lib.ptr(F)))
    folded = F[:nloc].copy()
    np.add.at(folded, owner, F[nloc:])
    tol = 1e-9 if prec == "fp64" else 1e-5
    assert abs(E[0] - ref["energy"]) < tol * nloc
    assert np.abs(folded - ref["force"]).max() < tol
    assert np.abs(V.reshape(3, 3, order="F") - ref["virial"]).max() < tol * 10
    # a pair descriptor centred on a local atom gives half its energy to its ghost
    # partner (local_e(ci(n)) += e fc / size(ci)); folded back, the periodic local
    # energies are recovered
    le = LE[:nloc].copy()
    np.add.at(le, owner, LE[nloc:])
    assert np.abs(le - ref["local_energy"]).max() < tol
    assert abs(LE.sum() - E[0]) < tol * nloc


def test_lammps_path_empty_region(tmp_path):
    from quip_gb300.potential import Potential
    pot = Potential(param_filename=sic_model(tmp_path))
    E = np.ones(1)
    F = np.ones((3, 3))
    lat = np.eye(3).ravel() * 10
    Z = np.array([14, 14, 14], np.int32)
    pos = np.zeros((3, 3))
    _lib.check(pot._L.gapgpu_calc_lammps(pot._ctx, 0, 3, _lib.ptr(Z), 0, None, None, None, _lib.ptr(lat), _lib.ptr(pos),
                                         _lib.ptr(E), None, None, None, _lib.ptr(F)))
    assert E[0] == 0.0 and np.all(F == 0.0)


def test_lammps_path_rejects_an_asymmetric_list(tmp_path):
    """A local-local pair listed for one atom only: the reverse-pair index finds no partner
    for the other direction and the call fails with its error, before any force is
    gathered."""
    from quip_gb300.potential import Potential
    path = sic_model(tmp_path)
    pot = Potential(param_filename=path, precision="fp64")
    at = models.random_triclinic(60, rng=np.random.default_rng(32))
    pos, Z, num, neigh, owner = _lammps_view(at, pot.cutoff())
    n, nloc = len(pos), len(at)
    first = [k for k in range(num[0]) if neigh[k] - 1 < nloc]   # local neighbours of atom 0
    assert first
    neigh = np.delete(neigh, first[-1])
    num = num.copy()
    num[0] -= 1
    ilist = np.arange(nloc, dtype=np.int32)
    lat = np.asfortranarray(at.lattice).ravel(order="F").copy()
    E, F, V = np.zeros(1), np.zeros((n, 3)), np.zeros(9)
    with pytest.raises(_lib.GapGpuError) as e:
        _lib.check(pot._L.gapgpu_calc_lammps(pot._ctx, nloc, n - nloc, _lib.ptr(Z), nloc, _lib.ptr(ilist), _lib.ptr(num),
                                             _lib.ptr(neigh), _lib.ptr(lat), _lib.ptr(np.ascontiguousarray(pos)),
                                             _lib.ptr(E), None, _lib.ptr(V), None, _lib.ptr(F)))
    assert "symmetric" in str(e.value)
