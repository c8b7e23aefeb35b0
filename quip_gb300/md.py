"""Device-resident velocity-Verlet MD of many replicas (gapgpu_md_* of libgapgpu).

Mirrors DynamicalSystem (src/libAtoms/DynamicalSystem.f95: advance_verlet1 :1814-2132,
advance_verlet2 :2159-2383) as DynamicalSystem_run drives it
(src/Potentials/Potential.f95:2304-2370), with the connection kept on a skin
(Connection.f95:1086-1125).  Units are QUIP's: positions in A, time in fs, energies in
eV, masses in eV fs^2 / A^2 (amu * MASSCONVERT, src/libAtoms/Units.f95:68).
Positions, velocities, forces and neighbour lists stay on the GPU between steps.
"""
import numpy as np

from . import _lib
from .models import MASS

# Units.f95:56-69 (restated): MASSCONVERT = 1/ELECTRONMASS_GPERMOL * HARTREE * AU_FS^2 / BOHR^2
_ELECTRONMASS_GPERMOL = 5.48579903e-4
_HARTREE = 27.2113961
_BOHR = 0.529177249
_HBAR_EVSEC = 6.5821220e-16
_AU_FS = 1.0 / (_HARTREE / _HBAR_EVSEC) * 1e15
MASSCONVERT = 1.0 / _ELECTRONMASS_GPERMOL * _HARTREE * _AU_FS * _AU_FS / (_BOHR * _BOHR)
BOLTZMANN_K = 8.617385e-5  # eV / K


def masses(numbers):
    """Per-atom masses in QUIP's internal units."""
    return np.array([MASS[int(z)] for z in numbers], dtype=np.float64) * MASSCONVERT


def maxwell_boltzmann(numbers, temperature, seed=0):
    """Velocities (N,3) in A/fs drawn from Maxwell-Boltzmann at `temperature` K, with the
    centre-of-mass momentum removed (DynamicalSystem.f95:1678 zero_momentum)."""
    rng = np.random.default_rng(seed)
    m = masses(numbers)
    v = rng.normal(size=(len(numbers), 3)) * np.sqrt(BOLTZMANN_K * temperature / m)[:, None]
    p = (m[:, None] * v).sum(axis=0)
    return v - p / m.sum()


def kinetic_energy(velo, m):
    return 0.5 * float(np.sum(m[:, None] * velo * velo))


class MDReplicas:
    """nstruct independent replicas integrated together on the GPU.

    MDReplicas(potential, replicas, dt=1.0, skin=0.5, temperature=None, seed=0)
    ``replicas`` is a list of Atoms; initial velocities come from
    ``atoms.arrays['velo']`` or, if absent, from Maxwell-Boltzmann at ``temperature``."""

    def __init__(self, potential, replicas, dt=1.0, skin=0.5, temperature=None, seed=0):
        L = _lib.load()
        self._L = L
        self.potential = potential
        self.replicas = replicas
        self.n_atoms = np.array([len(a) for a in replicas], dtype=np.int32)
        self.numbers = np.concatenate([a.numbers for a in replicas]).astype(np.int32)
        self.mass = masses(self.numbers)
        pos = np.ascontiguousarray(np.concatenate([a.positions for a in replicas]), dtype=np.float64)
        velo = []
        for k, a in enumerate(replicas):
            if "velo" in a.arrays:
                velo.append(np.asarray(a.arrays["velo"], dtype=np.float64))
            else:
                if temperature is None:
                    raise ValueError("give initial velocities (arrays['velo']) or a temperature")
                velo.append(maxwell_boltzmann(a.numbers, temperature, seed=seed + k))
        velo = np.ascontiguousarray(np.concatenate(velo), dtype=np.float64)
        lat = np.ascontiguousarray(np.concatenate([np.asfortranarray(a.lattice).ravel(order="F") for a in replicas]))
        pbc = np.ascontiguousarray(np.concatenate([np.asarray(a.pbc, dtype=np.int32).reshape(3) for a in replicas]))
        h = _lib.ctypes.c_void_p()
        _lib.check(L.gapgpu_md_create(potential._model, _lib.PRECISIONS[potential.precision], len(replicas),
                                      _lib.ptr(self.n_atoms), _lib.ptr(pos), _lib.ptr(velo), _lib.ptr(self.mass),
                                      _lib.ptr(self.numbers), _lib.ptr(lat), _lib.ptr(pbc), float(dt), float(skin),
                                      _lib.ctypes.byref(h)))
        self._md = h
        self.dt, self.skin = dt, skin

    def __del__(self):
        L = getattr(self, "_L", None)
        if L is not None and getattr(self, "_md", None):
            L.gapgpu_md_destroy(self._md)
            self._md = None

    def context(self):
        return self._L.gapgpu_md_context(self._md)

    def set_stream(self, cuda_stream):
        _lib.check(self._L.gapgpu_context_set_stream(self.context(), _lib.ctypes.c_void_p(cuda_stream)))

    def set_option(self, key, value):
        """Options of the replicas' context (gapgpu_context_set_option), as Potential.set_option."""
        _lib.check(self._L.gapgpu_context_set_option(self.context(), key.encode(), int(value)))

    def step(self, nsteps=1):
        _lib.check(self._L.gapgpu_md_step(self._md, int(nsteps)))

    def state(self):
        n = int(self.n_atoms.sum())
        pos, velo, force = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
        E = np.zeros(len(self.n_atoms))
        V = np.zeros((len(self.n_atoms), 9))
        _lib.check(self._L.gapgpu_md_state(self._md, _lib.ptr(pos), _lib.ptr(velo), _lib.ptr(force), _lib.ptr(E),
                                           _lib.ptr(V)))
        off = np.concatenate([[0], np.cumsum(self.n_atoms)])
        ke = np.array([kinetic_energy(velo[off[s]:off[s + 1]], self.mass[off[s]:off[s + 1]])
                       for s in range(len(self.n_atoms))])
        return {"pos": pos, "velo": velo, "force": force, "energy": E, "virial": V.reshape(-1, 3, 3).transpose(0, 2, 1),
                "kinetic": ke, "offsets": off}

    def neighbours(self):
        """The list the replicas' context holds now (built at cutoff + skin, its distances
        refreshed while it is kept): (offsets, j, shift, r) over all replicas' atoms."""
        L, ctx = self._L, self.context()
        n = int(self.n_atoms.sum())
        off = np.zeros(n + 1, np.int32)
        tot = _lib.ctypes.c_int64()
        _lib.check(L.gapgpu_context_neighbours(ctx, _lib.ptr(off), None, None, None, 0, _lib.ctypes.byref(tot)))
        j = np.zeros(tot.value, np.int32)
        sh = np.zeros((tot.value, 3), np.int32)
        r = np.zeros(tot.value)
        _lib.check(L.gapgpu_context_neighbours(ctx, _lib.ptr(off), _lib.ptr(j), _lib.ptr(sh), _lib.ptr(r), tot.value,
                                               _lib.ctypes.byref(tot)))
        return off, j, sh, r

    def counters(self):
        s, r, g = _lib.ctypes.c_int64(), _lib.ctypes.c_int64(), _lib.ctypes.c_int64()
        _lib.check(self._L.gapgpu_md_counters(self._md, _lib.ctypes.byref(s), _lib.ctypes.byref(r), _lib.ctypes.byref(g)))
        return {"steps": s.value, "rebuilds": r.value, "graph_replays": g.value}
