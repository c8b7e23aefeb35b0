"""Potential: the host-side mirror of QUIP's Potential API for the GAP path.

Mirrors quippy's ``Potential`` (quippy/quippy/potential.py:64-108 init, :177-325
calculate) and the Fortran ``potential_Filename_Initialise`` /
``potential_calc(pot, at, energy=, force=, virial=, local_energy=, local_virial=,
args_str=)`` (src/Potentials/Potential.f95:438-468, :803-996) for a GAP parameter file.
Every number is computed by libgapgpu.so on the GPU; this module only moves arrays.
"""
import os
import re

import numpy as np

from . import _lib
from .atoms import Atoms


def _epc_name(args_str):
    """The property name of energy_per_coordinate=<name> in a calc args string, or None."""
    m = re.search(r"(?:^|\s)energy_per_coordinate=(\S+)", args_str or "")
    return m.group(1) if m else None


def _variance_request(args_str):
    """(name of local_gap_variance=<name> or None, print_gap_variance given true)."""
    m = re.search(r"(?:^|\s)local_gap_variance=(\S+)", args_str or "")
    p = re.search(r"(?:^|\s)print_gap_variance(?:=(\S+))?(?:\s|$)", args_str or "")
    printed = bool(p) and (p.group(1) is None or p.group(1) in ("T", "t", "true", "True", "1"))
    return (m.group(1) if m else None), printed


def _init_args_from_xml(xml):
    """Default init args from the first <Potential init_args=...> tag (Potential.f95:525-538)."""
    m = re.search(r'<Potential[^>]*init_args="([^"]*)"', xml)
    return m.group(1) if m else "IP GAP"


def _key_val_str(args):
    """calc_args as an args string: a dict becomes key=value pairs (logicals as T/F)."""
    if args is None:
        return ""
    if isinstance(args, dict):
        fmt = lambda v: ("T" if v else "F") if isinstance(v, bool) else str(v)  # noqa: E731
        return " ".join("%s=%s" % (k, fmt(v)) for k, v in args.items())
    return str(args)


class Potential:
    """GAP potential evaluated on a GB300.

    Potential(args_str="IP GAP label=...", param_filename="gap.xml", precision="fp64")

    ``precision`` is "fp64" (plain path, matches the reference within 1e-8 eV/atom
    and 1e-7 eV/A) or a mixed path (FP32 SOAP, tensor-core kernel GEMMs): "bf16x3"
    (split-BF16, three products), "tf32" (TF32 operands) or "fp16" (FP16 operands where
    the model allows it -- the same 10-bit mantissas as TF32 at twice its rate -- else TF32).
    """

    def __init__(self, args_str="", pot1=None, pot2=None, param_str=None, param_filename=None, atoms=None,
                 calculation_always_required=False, calc_args=None, add_arrays=None, add_info=None,
                 precision="fp64", **kwargs):
        # quippy's signature (quippy/quippy/potential.py:64-108), plus the GPU precision
        if pot1 is not None or pot2 is not None:
            raise ValueError("sums of potentials (pot1, pot2) are outside this library: it evaluates 'IP GAP'")
        if (param_filename is None) == (param_str is None):
            raise ValueError("give exactly one of param_filename / param_str")
        if param_filename is not None:
            with open(param_filename) as f:
                xml = f.read()
            base = os.path.dirname(os.path.abspath(param_filename))
        else:
            xml, base = param_str, os.getcwd()
        if not args_str.strip():
            args_str = _init_args_from_xml(xml)
        toks = args_str.split()
        if "GAP" not in toks:
            raise ValueError("only 'IP GAP' potentials are handled by this library: %r" % args_str)
        self.args_str = args_str
        self.param_filename = param_filename
        self.precision = precision
        L = _lib.load()
        self._L = L
        h = _lib.ctypes.c_void_p()
        xb = xml.encode()
        _lib.check(L.gapgpu_model_create(xb, len(xb), args_str.encode(), base.encode(), _lib.ctypes.byref(h)))
        self._model = h
        c = _lib.ctypes.c_void_p()
        _lib.check(L.gapgpu_context_create(self._model, _lib.PRECISIONS[precision], _lib.ctypes.byref(c)))
        self._ctx = c
        self.results = {}
        self.extra_results = {"config": {}, "atoms": {}}
        self.calc_args = _key_val_str(calc_args)
        self.calculation_always_required = calculation_always_required
        self.add_arrays, self.add_info = add_arrays, add_info
        if atoms is not None:
            atoms.calc = self

    def __del__(self):
        L = getattr(self, "_L", None)
        if L is None:
            return
        if getattr(self, "_ctx", None):
            L.gapgpu_context_destroy(self._ctx)
            self._ctx = None
        if getattr(self, "_model", None):
            L.gapgpu_model_destroy(self._model)
            self._model = None

    # ------------------------------------------------------------------ info
    def cutoff(self):
        v = _lib.ctypes.c_double()
        _lib.check(self._L.gapgpu_model_cutoff(self._model, _lib.ctypes.byref(v)))
        return v.value

    def info(self):
        n = _lib.ctypes.c_int()
        dims = (_lib.ctypes.c_int * 64)()
        ns = (_lib.ctypes.c_int * 64)()
        _lib.check(self._L.gapgpu_model_info(self._model, _lib.ctypes.byref(n), dims, ns, 64))
        return [(dims[k], ns[k]) for k in range(n.value)]

    def n_coordinates(self):
        return len(self.info())

    def timings(self):
        ms = (_lib.ctypes.c_double * 7)()
        k = self._L.gapgpu_context_timings(self._ctx, ms, 7)
        names = ["neighbours", "soap_fwd", "gemm", "soap_bwd", "pair2b", "reduce", "total"]
        return dict(zip(names[:k], list(ms)[:k]))

    def launches(self):
        v = _lib.ctypes.c_int64()
        _lib.check(self._L.gapgpu_context_launches(self._ctx, _lib.ctypes.byref(v)))
        return v.value

    # ------------------------------------------------------------------ calc
    @staticmethod
    def _arrays(at):
        pos = np.ascontiguousarray(at.positions, dtype=np.float64)
        Z = np.ascontiguousarray(at.numbers, dtype=np.int32)
        lat = np.asfortranarray(at.lattice, dtype=np.float64).ravel(order="F").copy()
        pbc = np.ascontiguousarray(np.asarray(at.pbc, dtype=np.int32).reshape(3))
        return pos, Z, lat, pbc

    def calc(self, at, energy=True, force=True, virial=True, local_energy=False, local_virial=False, args_str="",
             atom_mask=None):
        """potential_calc: returns a dict with the requested quantities.

        energy (float), force (N,3), virial (3,3), local_energy (N,), local_virial (N,3,3).
        ``atom_mask`` is the logical property that args_str atom_mask_name names.
        args_str "energy_per_coordinate=<name>" adds out[<name>] (one value per coordinate,
        IPModel_GAP.f95:462,570); "only_descriptor=<k>" evaluates only coordinate k;
        "local_gap_variance=<name>" adds out[<name>] (per-atom variance estimate) and, with
        forces, out["gap_variance_gradient"] (N,3); "print_gap_variance=T" prints every
        descriptor instance's variance (IPModel_GAP.f95:464-488, 506-516).  The variance
        needs gap_variance_regularisation in the potential's init args."""
        pos, Z, lat, pbc = self._arrays(at)
        n = len(pos)
        E = np.zeros(1)
        F = np.zeros((n, 3)) if force else None
        V = np.zeros(9) if virial else None
        LE = np.zeros(n) if local_energy else None
        LV = np.zeros((n, 9)) if local_virial else None
        mask = None if atom_mask is None else np.ascontiguousarray(atom_mask, dtype=np.int32)
        _lib.check(self._L.gapgpu_calc(self._ctx, n, _lib.ptr(pos), _lib.ptr(Z), _lib.ptr(lat), _lib.ptr(pbc),
                                       _lib.ptr(mask), _lib.ptr(E) if energy else None, _lib.ptr(LE), _lib.ptr(F),
                                       _lib.ptr(V), _lib.ptr(LV), args_str.encode()))
        out = {}
        if energy:
            out["energy"] = float(E[0])
        if force:
            out["force"] = F
        if virial:
            out["virial"] = V.reshape(3, 3, order="F")
        if local_energy:
            out["local_energy"] = LE
        if local_virial:
            out["local_virial"] = LV.reshape(n, 3, 3).transpose(0, 2, 1)
        name = _epc_name(args_str)
        if name:
            out[name] = self._energy_per_coordinate(1)[0]
        vname, vprint = _variance_request(args_str)
        if vname or vprint:
            grad = force or virial or local_virial
            lv = np.zeros(n)
            gv = np.zeros((n, 3)) if grad else None
            _lib.check(self._L.gapgpu_gap_variance(self._ctx, _lib.ptr(lv), _lib.ptr(gv), n))
            if vname:
                out[vname] = lv
                if grad:
                    out["gap_variance_gradient"] = gv
            if vprint:
                self._print_gap_variance()
        self.results = out
        return out

    def gap_variance_instances(self, coordinate):
        """The variance of every descriptor instance of a coordinate (0-based) in the last
        calc that requested the variance: dict variance, fc2, atom_i, atom_j."""
        cnt = _lib.ctypes.c_int()
        _lib.check(self._L.gapgpu_gap_variance_instances(self._ctx, coordinate, None, None, None, None, 0,
                                                          _lib.ctypes.byref(cnt)))
        k = cnt.value
        v, f2 = np.zeros(k), np.zeros(k)
        ai, aj = np.zeros(k, np.int32), np.zeros(k, np.int32)
        _lib.check(self._L.gapgpu_gap_variance_instances(self._ctx, coordinate, _lib.ptr(v), _lib.ptr(f2), _lib.ptr(ai),
                                                          _lib.ptr(aj), k, _lib.ctypes.byref(cnt)))
        return dict(variance=v, fc2=f2, atom_i=ai, atom_j=aj)

    def _print_gap_variance(self):
        """print_gap_variance: one line per descriptor instance, as IPModel_GAP.f95:506-516
        prints them (atoms 1-based)."""
        label = re.search(r"label=(\S+)", self.args_str)
        label = label.group(1) if label else ""
        for k in range(self.n_coordinates()):
            d = self.gap_variance_instances(k)
            if len(d["variance"]) == 0:
                print("GAP_VARIANCE potential %s descriptor %d not found" % (label, k + 1))
            for i, (v, f2, a, b) in enumerate(zip(d["variance"], d["fc2"], d["atom_i"], d["atom_j"])):
                print("GAP_VARIANCE potential %s descriptor %d var( %d ) = %.16g * %.16g cutoff" % (label, k + 1, i + 1, v,
                                                                                                     f2))
                print("GAP_VARIANCE potential %s descriptor %d ii( %d ) = %s" % (label, k + 1, i + 1,
                                                                                " ".join(str(x + 1) for x in (a, b) if x >= 0)))

    def _energy_per_coordinate(self, nstruct):
        ncoord = self.n_coordinates()
        buf = np.zeros(nstruct * ncoord)
        cnt = _lib.ctypes.c_int()
        _lib.check(self._L.gapgpu_energy_per_coordinate(self._ctx, _lib.ptr(buf), len(buf), _lib.ctypes.byref(cnt)))
        return buf.reshape(nstruct, ncoord)

    def calc_batch(self, structures, args_str=""):
        """Energies, forces and virials of many independent structures in one GPU pass
        (gapgpu_calc_batch).  Returns a list of dicts energy / force (N,3) / virial (3,3),
        one per structure, each bit-identical to ``calc`` of that structure alone."""
        ns = np.array([len(a) for a in structures], dtype=np.int32)
        if len(ns) == 0:
            return []
        pos = np.ascontiguousarray(np.concatenate([a.positions for a in structures]), dtype=np.float64)
        Z = np.ascontiguousarray(np.concatenate([a.numbers for a in structures]), dtype=np.int32)
        lat = np.ascontiguousarray(np.concatenate([np.asfortranarray(a.lattice, dtype=np.float64).ravel(order="F")
                                                   for a in structures]))
        pbc = np.ascontiguousarray(np.concatenate([np.asarray(a.pbc, dtype=np.int32).reshape(3) for a in structures]))
        E = np.zeros(len(ns))
        F = np.zeros((len(pos), 3))
        V = np.zeros((len(ns), 9))
        _lib.check(self._L.gapgpu_calc_batch(self._ctx, len(ns), _lib.ptr(ns), _lib.ptr(pos), _lib.ptr(Z), _lib.ptr(lat),
                                             _lib.ptr(pbc), _lib.ptr(E), _lib.ptr(F), _lib.ptr(V), args_str.encode()))
        name = _epc_name(args_str)
        epc = self._energy_per_coordinate(len(ns)) if name else None
        out, a0 = [], 0
        for s, n in enumerate(ns):
            out.append({"energy": float(E[s]), "force": F[a0:a0 + n], "virial": V[s].reshape(3, 3, order="F")})
            if name:
                out[-1][name] = epc[s]
            a0 += n
        return out

    def set_option(self, key, value):
        """Context options (gapgpu_context_set_option): graphs (CUDA-graph replay of
        repeated shapes), timing, priority, autotune, pairs (CTA-pair GEMM tiles),
        gemm1_f16 / gemm2_f16 (the first / second GEMM with FP16 operands on the TF32 path),
        soap_bwd (1: the SOAP backward with one thread per pair where the basis has an
        instance, 0: one block per centre), soap_fwd (1: the fixed-size SOAP forward where
        the basis has an instance, 0: the generic one)."""
        _lib.check(self._L.gapgpu_context_set_option(self._ctx, key.encode(), int(value)))

    def footprint(self, n_atoms, mean_neighbours=60.0):
        """Estimated device bytes of one evaluation of n_atoms atoms."""
        b = _lib.ctypes.c_int64()
        _lib.check(self._L.gapgpu_model_footprint(self._model, _lib.PRECISIONS[self.precision], int(n_atoms),
                                                  float(mean_neighbours), _lib.ctypes.byref(b)))
        return b.value

    # the calculator interface of quippy's Potential (quippy/quippy/potential.py:44-62, :177-357)
    implemented_properties = ["energy", "free_energy", "forces", "stress", "stresses", "energies"]
    extra_properties = ["virial", "local_virial", "local_energy"]
    _default_properties = ["energy", "forces"]
    calc_args = ""

    def get_default_properties(self):
        return list(self._default_properties)

    def set_default_properties(self, properties):
        self._default_properties = list(properties)

    def calculate(self, atoms, properties=None, vol_per_atom=None):
        """ASE-calculator view, as quippy's (quippy/quippy/potential.py:177-325).  The
        properties asked for are added to the defaults (energy, forces).  Results: energy,
        free_energy, forces (N,3) and stress = -virial / volume as a 6-vector in Voigt order
        (xx, yy, zz, yz, xz, xy; potential.py:279-284); with "energies" the local energies;
        with "stresses" the per-atom stresses -local_virial / atomic volume, the atomic
        volume being `vol_per_atom` (the name of a per-atom array of `atoms`, or a number),
        else volume / N (potential.py:296-313).  extra_results keeps the virial (3,3) and
        the local energies (N,) and local virials (9,N, Fortran layout) as quippy does."""
        props = set(self.get_default_properties()) | set(properties or ())
        for prop in props:
            if prop not in self.implemented_properties + self.extra_properties:
                raise RuntimeError("Don't know how to calculate property '%s'" % prop)
        want_le = bool(props & {"energies", "local_energy"})
        want_lv = bool(props & {"stresses", "local_virial"})
        r = self.calc(atoms, energy=True, force=True, virial=True, local_energy=want_le, local_virial=want_lv,
                      args_str=self.calc_args)
        res = {"energy": r["energy"], "free_energy": r["energy"], "forces": r["force"]}
        s = -r["virial"] / atoms.volume()
        res["stress"] = np.array([s[0, 0], s[1, 1], s[2, 2], s[1, 2], s[0, 2], s[0, 1]])
        extra = {"config": {"virial": np.array(r["virial"], copy=True)}, "atoms": {}}
        if want_le:
            res["energies"] = r["local_energy"]
            extra["atoms"]["local_energy"] = np.array(r["local_energy"], copy=True)
        if want_lv:
            lv = np.asarray(r["local_virial"])                       # (N, 3, 3)
            extra["atoms"]["local_virial"] = lv.transpose(0, 2, 1).reshape(len(lv), 9).T.copy()
            if vol_per_atom is None:
                v_atom = atoms.volume() / len(atoms)
            elif isinstance(vol_per_atom, str) and vol_per_atom in atoms.arrays:
                v_atom = np.asarray(atoms.arrays[vol_per_atom], dtype=np.float64).reshape(-1, 1, 1)
            else:
                try:
                    v_atom = float(vol_per_atom)
                except (TypeError, ValueError):
                    raise ValueError("volume_per_atom: not found in atoms.arrays and not a number")
            res["stresses"] = -lv / v_atom
        self.results = res
        self.extra_results = extra
        return res

    def get_potential_energy(self, atoms):
        return self.calc(atoms, force=False, virial=False)["energy"]

    def get_forces(self, atoms):
        return self.calc(atoms, energy=False, virial=False)["force"]

    def get_stress(self, atoms):
        """-virial / volume in Voigt order, as ASE's get_stress."""
        return self.calculate(atoms, ["stress"])["stress"]

    def get_virial(self, atoms):
        self.calculate(atoms, ["stress"])
        return self.extra_results["config"]["virial"]

    def get_energies(self, atoms):
        return self.calculate(atoms, ["energies"])["energies"]

    get_local_energy = get_energies

    def get_stresses(self, atoms, vol_per_atom=None):
        return self.calculate(atoms, ["stresses"], vol_per_atom=vol_per_atom)["stresses"]

    def get_local_virial(self, atoms):
        """(9, N): each atom's virial as 9 values in column-major order."""
        self.calculate(atoms, ["local_virial"])
        return self.extra_results["atoms"]["local_virial"]

    # ------------------------------------------------------------------ auxiliaries
    def neighbours(self, at, cutoff=None):
        """QUIP-semantics neighbour list built on the GPU: (offsets, j, shift)."""
        pos, Z, lat, pbc = self._arrays(at)
        n = len(pos)
        rc = self.cutoff() if cutoff is None else cutoff
        off = np.zeros(n + 1, np.int32)
        tot = _lib.ctypes.c_int64()
        _lib.check(self._L.gapgpu_neighbours(self._ctx, n, _lib.ptr(pos), _lib.ptr(lat), _lib.ptr(pbc), rc,
                                             _lib.ptr(off), None, None, 0, _lib.ctypes.byref(tot)))
        j = np.zeros(tot.value, np.int32)
        sh = np.zeros((tot.value, 3), np.int32)
        _lib.check(self._L.gapgpu_neighbours(self._ctx, n, _lib.ptr(pos), _lib.ptr(lat), _lib.ptr(pbc), rc,
                                             _lib.ptr(off), _lib.ptr(j), _lib.ptr(sh), tot.value, _lib.ctypes.byref(tot)))
        return off, j, sh

    def descriptors(self, at, coordinate=0):
        """SOAP descriptors of every centre of the given coordinate (n_centres, dim)."""
        pos, Z, lat, pbc = self._arrays(at)
        dim = self.info()[coordinate][0]
        q = np.zeros((len(pos), dim))
        nc = _lib.ctypes.c_int()
        _lib.check(self._L.gapgpu_descriptors(self._ctx, coordinate, len(pos), _lib.ptr(pos), _lib.ptr(Z),
                                              _lib.ptr(lat), _lib.ptr(pbc), _lib.ptr(q), q.size,
                                              _lib.ctypes.byref(nc)))
        return q[:nc.value]


__all__ = ["Potential", "Atoms"]
