"""ctypes front end of the FP64 CPU oracle (oracle/gap_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by
the CPU-baseline legs of bench.py.  The product path (quip_gb300) never imports it.

This module also holds the oracle's own GAP XML reader.  It is deliberately
independent of the product's C++ reader so that the two parse the same file
separately.  It follows the reference's reader: IPModel_GAP_read_params_xml
(src/Potentials/IPModel_GAP.f95:618-944) for GAP_params/GAP_data/e0, and the
gpSparse/gpCoordinates/sparseX layout documented by quippy/quippy/gap_tools.py:17-75
and tests/test_gapfit.py:154-170 (sparseX_filename holds M*D values, one per line).
"""
import ctypes
import os
import re
import subprocess
import xml.etree.ElementTree as ET

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

_lib = None


def build():
    """Compile liboracle.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        d, i, l, v = ctypes.c_double, ctypes.c_int, ctypes.c_long, ctypes.c_void_p
        P = ctypes.POINTER
        L.oracle_neighbours.restype = l
        L.oracle_neighbours.argtypes = [i, P(d), P(d), P(i), d, P(i), P(i), P(i), P(d), P(d), l]
        L.oracle_model_new.restype = v
        L.oracle_model_free.argtypes = [v]
        L.oracle_model_set_e0.argtypes = [v, i, d]
        L.oracle_model_set_E_scale.argtypes = [v, d]
        L.oracle_soap_dim.restype = i
        L.oracle_soap_dim.argtypes = [P(d), P(i)]
        L.oracle_model_add_soap.restype = i
        L.oracle_model_add_soap.argtypes = [v, P(d), P(i), i, P(d), i, i, P(d), P(d), P(d)]
        L.oracle_model_add_distance_2b.restype = i
        L.oracle_model_add_distance_2b.argtypes = [v, d, d, i, i, i, P(d), i, P(d), P(d), P(d)]
        L.oracle_model_cutoff.restype = d
        L.oracle_model_cutoff.argtypes = [v]
        L.oracle_soap.restype = i
        L.oracle_soap.argtypes = [P(d), P(i), i, P(d), P(i), P(d), P(i), d, P(d), l, P(d), P(i), l, P(l)]
        L.oracle_gap_calc.restype = i
        L.oracle_gap_calc.argtypes = [v, i, P(d), P(i), P(d), P(i), P(i), P(d), P(d), P(d), P(d), P(d), i]
        L.oracle_gap_calc_ex.restype = i
        L.oracle_gap_calc_ex.argtypes = [v, i, P(d), P(i), P(d), P(i), P(i), i, i, P(d), P(d), P(d), P(d), P(d), P(d), i]
        L.oracle_model_n_coordinates.restype = i
        L.oracle_model_n_coordinates.argtypes = [v]
        L.oracle_model_init_variance.restype = i
        L.oracle_model_init_variance.argtypes = [v, d]
        L.oracle_gap_variance.restype = l
        L.oracle_gap_variance.argtypes = [v, i, P(d), P(i), P(d), P(i), P(i), i, i, P(d), P(d), P(d), l, i]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if a is not None else None


# ------------------------------------------------------------------ descriptor strings
def parse_args(s):
    """key=value parser with {..} and quoted values (ParamReader.f95 semantics)."""
    out = {}
    toks = re.findall(r'(\S+?)=(\{[^}]*\}|"[^"]*"|\S+)|(\S+)', s)
    for k, v, bare in toks:
        if bare:
            out[bare] = True
            continue
        v = v.strip()
        if v.startswith("{") or v.startswith('"'):
            v = v[1:-1].strip()
        out[k] = v
    return out


def _ints(v):
    return [int(x) for x in str(v).replace(",", " ").split()]


def _bool(v):
    return str(v).strip().upper() in ("T", "TRUE", "1", ".TRUE.")


def soap_param_arrays(desc):
    """Descriptor string dict -> (fp, ip) arrays of oracle_soap / add_soap."""
    g = lambda k, dflt: desc.get(k, dflt)
    sigma = float(desc.get("atom_sigma", desc.get("atom_gaussian_width", 1.0)))
    n_species = int(g("n_species", 1))
    species_Z = _ints(g("species_Z", " ".join(["0"] * n_species)))
    Zs = _ints(g("Z", "0"))
    n_Z = int(g("n_Z", len(Zs)))
    fp = np.array([float(g("cutoff", 0.0)), float(g("cutoff_transition_width", 0.5)), sigma,
                   float(g("central_weight", 1.0)), float(g("covariance_sigma0", 0.0)),
                   float(g("basis_error_exponent", 10.0))], dtype=np.float64)
    ip = np.array([int(g("l_max", 4)), int(g("n_max", 4)), n_species, n_Z, int(_bool(g("normalise", "T"))),
                   int(_bool(g("diagonal_radial", "F"))), int(_bool(g("central_reference_all_species", "F"))), 1]
                  + species_Z[:n_species] + Zs[:n_Z], dtype=np.int32)
    return fp, ip


# ------------------------------------------------------------------ structures
def neighbours(pos, lattice, pbc, cutoff):
    """QUIP-order full neighbour list: (offsets, j, shift, diff, r).
    pos (N,3); lattice (3,3) with COLUMNS = cell vectors (Fortran at%lattice)."""
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    lat = np.asfortranarray(lattice, dtype=np.float64).ravel(order="F").copy()
    pbc = np.ascontiguousarray(np.asarray(pbc, dtype=np.int32).reshape(3))
    n = len(pos)
    off = np.zeros(n + 1, np.int32)
    L = lib()
    tot = L.oracle_neighbours(n, _dp(pos), _dp(lat), _ip(pbc), cutoff, _ip(off), None, None, None, None, 0)
    j = np.zeros(tot, np.int32); sh = np.zeros((tot, 3), np.int32)
    df = np.zeros((tot, 3)); r = np.zeros(tot)
    L.oracle_neighbours(n, _dp(pos), _dp(lat), _ip(pbc), cutoff, _ip(off), _ip(j), _ip(sh), _dp(df), _dp(r), tot)
    return off, j, sh, df, r


def soap(desc_str, pos, Z, lattice, pbc, grad=False, list_cutoff=0.0):
    """SOAP descriptors of every centre (and gradients): the quippy
    Descriptor.calc view (quippy/quippy/descriptors.py:165-235)."""
    desc = parse_args(desc_str)
    fp, ip = soap_param_arrays(desc)
    L = lib()
    dim = L.oracle_soap_dim(_dp(fp), _ip(ip))
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    Z = np.ascontiguousarray(Z, dtype=np.int32)
    lat = np.asfortranarray(lattice, dtype=np.float64).ravel(order="F").copy()
    pbc = np.ascontiguousarray(np.asarray(pbc, dtype=np.int32).reshape(3))
    n = len(pos)
    q = np.zeros((n, dim))
    ng = ctypes.c_long(0)
    if grad:
        L.oracle_soap(_dp(fp), _ip(ip), n, _dp(pos), _ip(Z), _dp(lat), _ip(pbc), list_cutoff, _dp(q), q.size, None,
                      None, 0, ctypes.byref(ng))
        # count pass for gradient entries
        cnt = ctypes.c_long(0)
        g = np.zeros((1, 3, dim)); gi = np.zeros((1, 2), np.int32)
        L.oracle_soap(_dp(fp), _ip(ip), n, _dp(pos), _ip(Z), _dp(lat), _ip(pbc), list_cutoff, _dp(q), q.size, _dp(g),
                      _ip(gi), 0, ctypes.byref(cnt))
        g = np.zeros((cnt.value, 3, dim)); gi = np.zeros((cnt.value, 2), np.int32)
        nd = L.oracle_soap(_dp(fp), _ip(ip), n, _dp(pos), _ip(Z), _dp(lat), _ip(pbc), list_cutoff, _dp(q), q.size,
                           _dp(g), _ip(gi), cnt.value, ctypes.byref(cnt))
        return q[:nd], g, gi
    nd = L.oracle_soap(_dp(fp), _ip(ip), n, _dp(pos), _ip(Z), _dp(lat), _ip(pbc), list_cutoff, _dp(q), q.size, None,
                       None, 0, ctypes.byref(ng))
    return q[:nd]


# ------------------------------------------------------------------ GAP XML
def read_gap_xml(path, label=None):
    """Parse a GAP XML file into a plain dict (oracle-side reader)."""
    base = os.path.dirname(os.path.abspath(path))
    root = ET.parse(path).getroot()
    gp_params = None
    for el in root.iter("GAP_params"):
        if label is None or el.attrib.get("label", "") == label:
            gp_params = el
            break
    if gp_params is None:
        raise ValueError("no GAP_params with label %r" % label)
    e0 = {}
    gd = gp_params.find("GAP_data")
    if gd is not None:
        if "e0" in gd.attrib:
            v = float(gd.attrib["e0"])
            e0 = {z: v for z in range(1, 117)}
        for e in gd.findall("e0"):
            e0[int(e.attrib["Z"])] = float(e.attrib["value"])
    coords = []
    sp = gp_params.find("gpSparse")
    for gc in sp.findall("gpCoordinates"):
        a = gc.attrib
        D = int(a["dimensions"])
        cov = int(a["covariance_type"])
        sx = gc.findall("sparseX")
        alpha = np.array([float(s.attrib["alpha"]) for s in sx])
        scut = np.array([float(s.attrib.get("sparseCutoff", 1.0)) for s in sx])
        M = len(sx)
        if "sparseX_filename" in a:
            X = np.fromfile(os.path.join(base, a["sparseX_filename"]), sep=" ").reshape(M, D)
        else:
            X = np.array([[float(v) for v in (s.text or "").split()] for s in sx]).reshape(M, D)
        theta = None
        th = gc.find("theta")
        if th is not None and th.text and th.text.strip():
            theta = np.array([float(v) for v in th.text.split()])
        desc = gc.find("descriptor").text.strip()
        coords.append(dict(desc_str=desc, desc=parse_args(desc), cov=cov, delta=float(a["signal_variance"]),
                           zeta=float(a.get("zeta", 1.0)), theta=theta, M=M, D=D, X=X, alpha=alpha, sc=scut))
    return dict(e0=e0, coords=coords, label=gp_params.attrib.get("label", ""))


class OracleModel:
    """A GAP model loaded into the oracle."""

    def __init__(self, parsed, E_scale=1.0):
        L = lib()
        self._h = L.oracle_model_new()
        for z, v in parsed["e0"].items():
            L.oracle_model_set_e0(self._h, z, v)
        L.oracle_model_set_E_scale(self._h, E_scale)
        for c in parsed["coords"]:
            kind = next(iter(c["desc"]))
            covfp = np.zeros(2 + max(1, c["D"]))
            covfp[0] = c["delta"]; covfp[1] = c["zeta"]
            if c["theta"] is not None:
                covfp[2:2 + len(c["theta"])] = c["theta"]
            X = np.ascontiguousarray(c["X"], dtype=np.float64)
            al = np.ascontiguousarray(c["alpha"], dtype=np.float64)
            sc = np.ascontiguousarray(c["sc"], dtype=np.float64)
            if kind == "soap":
                fp, ip = soap_param_arrays(c["desc"])
                rc = L.oracle_model_add_soap(self._h, _dp(fp), _ip(ip), c["cov"], _dp(covfp), c["M"], c["D"], _dp(X),
                                             _dp(al), _dp(sc))
                if rc != 0:
                    raise ValueError("SOAP dimension mismatch for %r" % c["desc_str"])
            elif kind == "distance_2b":
                d = c["desc"]
                L.oracle_model_add_distance_2b(self._h, float(d["cutoff"]), float(d.get("cutoff_transition_width", 0.5)),
                                               int(d.get("Z1", 0)), int(d.get("Z2", 0)), c["cov"], _dp(covfp), c["M"],
                                               _dp(X), _dp(al), _dp(sc))
            else:
                raise ValueError("descriptor %r not supported by the oracle" % kind)

    @classmethod
    def from_xml(cls, path, label=None, E_scale=1.0):
        return cls(read_gap_xml(path, label), E_scale)

    def cutoff(self):
        return lib().oracle_model_cutoff(self._h)

    def __del__(self):
        try:
            lib().oracle_model_free(self._h)
        except Exception:
            pass

    def init_variance(self, regularisation=0.001):
        """Variance estimate set-up, as the init arg gap_variance_regularisation
        (IPModel_GAP.f95:185-187): K_MM + regularisation * I factorised per coordinate."""
        if lib().oracle_model_init_variance(self._h, float(regularisation)) != 0:
            raise ValueError("K_MM + regularisation I is not positive definite")

    def variance(self, pos, Z, lattice, pbc=(1, 1, 1), mask=None, gradient=True, nthreads=0, only_descriptor=None):
        """local_gap_variance (N,), gap_variance_gradient (N,3) and the variance of every
        descriptor instance (IPModel_GAP.f95:464-488, 506-516)."""
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        n = len(pos)
        Z = np.ascontiguousarray(Z, dtype=np.int32)
        lat = np.asfortranarray(lattice, dtype=np.float64).ravel(order="F").copy()
        pbc = np.ascontiguousarray(np.asarray(pbc, dtype=np.int32).reshape(3))
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        lv = np.zeros(n)
        g = np.zeros((n, 3)) if gradient else None
        sel = only_descriptor is not None
        L = lib()
        args = (self._h, n, _dp(pos), _ip(Z), _dp(lat), _ip(pbc), _ip(m), int(sel), int(only_descriptor) if sel else 0,
                _dp(lv), _dp(g))
        ni = L.oracle_gap_variance(*args, None, 0, nthreads)
        if ni < 0:
            raise RuntimeError("oracle_gap_variance failed (variance not initialised?)")
        iv = np.zeros(ni)
        L.oracle_gap_variance(*args, _dp(iv), ni, nthreads)
        return dict(local_gap_variance=lv, gap_variance_gradient=g, instance_variance=iv)

    def calc(self, pos, Z, lattice, pbc=(1, 1, 1), mask=None, nthreads=0, only_descriptor=None):
        """E, local_e, F (N,3), virial (3,3), local_virial (N,3,3) and energy_per_coordinate
        (one value per coordinate: sum of e_i * covariance_cutoff, before E_scale, no e0).
        only_descriptor: the calc argument of that name (1-based coordinate; with more than
        one coordinate only that one is evaluated)."""
        pos = np.ascontiguousarray(pos, dtype=np.float64)
        n = len(pos)
        Z = np.ascontiguousarray(Z, dtype=np.int32)
        lat = np.asfortranarray(lattice, dtype=np.float64).ravel(order="F").copy()
        pbc = np.ascontiguousarray(np.asarray(pbc, dtype=np.int32).reshape(3))
        m = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        E = np.zeros(1); le = np.zeros(n); F = np.zeros((n, 3)); V = np.zeros(9); LV = np.zeros((n, 9))
        epc = np.zeros(lib().oracle_model_n_coordinates(self._h))
        sel = only_descriptor is not None
        rc = lib().oracle_gap_calc_ex(self._h, n, _dp(pos), _ip(Z), _dp(lat), _ip(pbc), _ip(m), int(sel),
                                      int(only_descriptor) if sel else 0, _dp(epc), _dp(E), _dp(le), _dp(F), _dp(V),
                                      _dp(LV), nthreads)
        if rc != 0:
            raise RuntimeError("oracle_gap_calc failed")
        return dict(energy=E[0], local_energy=le, force=F, virial=V.reshape(3, 3, order="F"),
                    local_virial=LV.reshape(n, 3, 3).transpose(0, 2, 1), energy_per_coordinate=epc)
