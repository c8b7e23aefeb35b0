"""CPU-side checks of the C ABI and the host logic (no GPU compute)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from quip_gb300 import _lib, models
from oracle import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    hdr = open(os.path.join(ROOT, "include", "gapgpu.h")).read()
    return sorted(set(re.findall(r"\b(gapgpu_\w+)\s*\(", hdr)))


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    declared = _declared_symbols()
    assert declared == sorted(_lib.EXPORTS)
    for s in declared:
        assert hasattr(L, s), s
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    for s in declared:
        assert re.search(r"\bT %s\b" % s, out), s


def test_package_exports_the_quippy_style_api():
    """The quippy-style entry points import from the package, as a quippy user writes them."""
    from quip_gb300 import Atoms, Potential, read_xyz, write_xyz
    for name in ("calc", "calculate", "calc_batch", "cutoff", "neighbours", "descriptors"):
        assert callable(getattr(Potential, name)), name
    assert callable(read_xyz) and callable(write_xyz) and Atoms is models.Atoms


def test_ase_view_matches_quippy_conventions():
    """The calculator interface of quippy's Potential (quippy/quippy/potential.py:44-62,
    :177-357): stress = -virial / volume in Voigt order (xx, yy, zz, yz, xz, xy), per-atom
    stresses = -local_virial / atomic volume, the virial (3,3) and local virials (9,N,
    Fortran layout) in extra_results, the getters, and the property checks.  Host logic
    only: calc is stubbed."""
    from quip_gb300 import Potential
    rng = np.random.default_rng(2)
    n = 4
    at = models.Atoms(np.full(n, 14), rng.uniform(0, 5, (n, 3)), lattice=np.diag([5.0, 6.0, 7.0]))
    at.arrays["vol"] = np.array([40.0, 50.0, 60.0, 60.0])
    V = rng.normal(size=(3, 3))
    LV = rng.normal(size=(n, 3, 3))
    pot = object.__new__(Potential)
    pot.calc = lambda a, **k: {"energy": -1.5, "force": np.ones((n, 3)), "virial": V,
                               "local_energy": np.arange(n, dtype=float), "local_virial": LV}
    assert pot.get_default_properties() == ["energy", "forces"]
    r = pot.calculate(at, ["stress", "energies", "stresses"])
    s = -V / 210.0
    np.testing.assert_allclose(r["stress"], [s[0, 0], s[1, 1], s[2, 2], s[1, 2], s[0, 2], s[0, 1]])
    np.testing.assert_allclose(r["stresses"], -LV / (210.0 / n))
    assert r["free_energy"] == r["energy"] == -1.5 and r["energies"].shape == (n,)
    np.testing.assert_array_equal(pot.extra_results["config"]["virial"], V)
    lv9 = pot.extra_results["atoms"]["local_virial"]
    assert lv9.shape == (9, n)
    for a in range(n):   # column a: atom a's virial, column-major
        np.testing.assert_array_equal(lv9[:, a].reshape(3, 3, order="F"), LV[a])
    np.testing.assert_allclose(pot.get_stresses(at, vol_per_atom=30.0), -LV / 30.0)
    np.testing.assert_allclose(pot.get_stresses(at, vol_per_atom="vol"), -LV / at.arrays["vol"][:, None, None])
    with pytest.raises(ValueError):
        pot.get_stresses(at, vol_per_atom="no_such_array")
    with pytest.raises(RuntimeError):
        pot.calculate(at, ["magnetic_moments"])
    np.testing.assert_allclose(pot.get_stress(at), r["stress"])
    np.testing.assert_array_equal(pot.get_virial(at), V)
    np.testing.assert_array_equal(pot.get_local_virial(at), lv9)
    np.testing.assert_array_equal(pot.get_energies(at), np.arange(n))
    np.testing.assert_array_equal(pot.get_local_energy(at), np.arange(n))
    pot.set_default_properties(["energy", "forces", "stress"])
    assert "stress" in pot.get_default_properties()


def test_quippy_constructor_arguments():
    """quippy's constructor keywords: a sum of potentials is refused; calc_args (a string,
    or a dict written as key=value with logicals as T/F) is the args string calculate()
    passes to calc, as quippy's calculator does."""
    from quip_gb300 import Potential
    from quip_gb300.potential import _key_val_str
    with pytest.raises(ValueError, match="sums of potentials"):
        Potential("Sum", pot1=object(), pot2=object())
    assert _key_val_str({"only_descriptor": 2, "do_calc_connect": True}) == "only_descriptor=2 do_calc_connect=T"
    assert _key_val_str(None) == "" and _key_val_str("a=1") == "a=1"
    seen = []
    pot = object.__new__(Potential)
    pot.calc_args = _key_val_str({"energy_per_coordinate": "epc"})
    pot.calc = lambda a, **k: (seen.append(k.get("args_str")),
                               {"energy": 0.0, "force": np.zeros((1, 3)), "virial": np.zeros((3, 3))})[1]
    at = models.Atoms([14], np.zeros((1, 3)), lattice=np.eye(3) * 5.0)
    pot.calculate(at)
    assert seen == ["energy_per_coordinate=epc"]


def test_constructor_runs_through_with_a_stub_library(monkeypatch):
    """The whole constructor, with the library calls answered by a stub (model and
    context created): quippy's keywords land where calculate() and ASE expect them."""
    from quip_gb300 import Potential, potential

    class _Stub:
        def __getattr__(self, name):
            return lambda *a: 0

    monkeypatch.setattr(potential._lib, "load", lambda *a, **k: _Stub())
    at = models.Atoms([14], np.zeros((1, 3)), lattice=np.eye(3) * 5.0)
    pot = Potential(param_filename=os.path.join(ROOT, "tests", "golden", "gap_water", "GAP.xml"),
                    calc_args={"only_descriptor": 1}, atoms=at, precision="tf32")
    assert pot.args_str.startswith("IP GAP label=") and pot.precision == "tf32"
    assert pot.calc_args == "only_descriptor=1" and at.calc is pot
    assert pot.extra_results == {"config": {}, "atoms": {}} and pot.results == {}


def test_bad_xml_is_rejected_before_device_use():
    L = _lib.load()
    h = ctypes.c_void_p()
    x = b"<GAP><GAP_params label='a'><gpSparse></GAP_params>"
    rc = L.gapgpu_model_create(x, len(x), b"", b".", ctypes.byref(h))
    assert rc == _lib.ERR_XML
    assert b"mismatched" in L.gapgpu_last_error() or b"parse" in L.gapgpu_last_error()


C_HOST = r"""
#include "gapgpu.h"
#include <stdio.h>
#include <string.h>
int main(void) {
    gapgpu_model* m = NULL;
    const char* xml = "<GAP><GAP_params label='a'><gpSparse></GAP_params>";
    int rc = gapgpu_model_create(xml, strlen(xml), "", ".", &m);
    printf("%d %s\n", rc, gapgpu_last_error());
    return (rc == GAPGPU_ERR_XML && m == NULL) ? 0 : 1;
}
"""


def test_header_serves_a_plain_c_host(tmp_path):
    """include/gapgpu.h compiles as strict C99 and a C program links against
    libgapgpu.so and gets a status and a message back (no GPU call)."""
    _lib.load()
    src = tmp_path / "host.c"
    src.write_text(C_HOST)
    exe = str(tmp_path / "host")
    build = lambda *a: subprocess.run(list(a), capture_output=True, text=True)  # noqa: E731
    r = build("gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
              str(src), "-L", os.path.dirname(_lib.LIB_PATH), "-lgapgpu",
              "-Wl,-rpath," + os.path.dirname(_lib.LIB_PATH), "-o", exe)
    assert r.returncode == 0, r.stderr
    r = build(exe)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("%d " % _lib.ERR_XML) and len(r.stdout.strip()) > 2


def test_unsupported_descriptor_is_rejected(tmp_path):
    L = _lib.load()
    p = models.write_gap_xml(str(tmp_path / "g.xml"),
                             [dict(desc_str="bispectrum_so4 cutoff=3.0 j_max=4", cov="dot_product", delta=1.0, zeta=2.0,
                                   X=np.ones((2, 5)), alpha=np.ones(2), sc=np.ones(2))])
    x = open(p, "rb").read()
    h = ctypes.c_void_p()
    rc = L.gapgpu_model_create(x, len(x), b"", str(tmp_path).encode(), ctypes.byref(h))
    assert rc == _lib.ERR_UNSUPPORTED


def _water_copy(tmp_path):
    src = os.path.join(ROOT, "tests", "golden", "gap_water")
    for f in os.listdir(src):
        if f.startswith("GAP.xml"):
            (tmp_path / f).write_bytes(open(os.path.join(src, f), "rb").read())
    return (tmp_path / "GAP.xml").read_text()


def _truncate(path, keep):
    lines = open(path).read().splitlines()[:keep]
    open(path, "w").write("\n".join(lines) + "\n")


SPX = "GAP.xml.sparseX.GAP_2018_10_7_60_14_59_24_970"
# (case, edit of the XML text and files, init_args, expected status, message fragment)
MODEL_CASES = [
    ("label", lambda x, d: x, "IP GAP label=nope", "ERR_XML", "no GAP_params stanza with label 'nope'"),
    ("missing sparseX file", lambda x, d: (os.remove(d / (SPX + "2")), x)[1], "", "ERR_XML", "cannot open sparseX file"),
    ("short sparseX file", lambda x, d: (_truncate(d / (SPX + "3"), 5), x)[1], "", "ERR_XML", "fewer than M*D"),
    ("signal_mean", lambda x, d: x.replace('signal_mean=".00000000000000000E+000"', 'signal_mean="0.5"', 1), "",
     "ERR_UNSUPPORTED", "signal_mean"),
    ("covariance_type", lambda x, d: x.replace('covariance_type="1"', 'covariance_type="3"', 1), "",
     "ERR_UNSUPPORTED", "covariance_type 3"),
    ("permutations", lambda x, d: x.replace('n_permutations="1"', 'n_permutations="2"', 1), "",
     "ERR_UNSUPPORTED", "permutations"),
    ("do_pca", lambda x, d: x.replace('<GAP_data do_core="F">', '<GAP_data do_core="F" do_pca="T">', 1), "",
     "ERR_UNSUPPORTED", "do_pca"),
    ("bad e0", lambda x, d: x.replace('<e0 Z="2" value=".00000000000000000E+000"/>', '<e0 Z="2" value="x"/>', 1), "",
     "ERR_XML", "bad e0 entry"),
    ("distance_2b dimensions", lambda x, d: x.replace('dimensions="1"', 'dimensions="2"', 1), "",
     "ERR_XML", "dimensions=1"),
    ("ard_se without theta", lambda x, d: x.replace("<theta>  0.10000000000000000E+001 </theta>", "", 1), "",
     "ERR_XML", "without theta"),
]


@pytest.mark.parametrize("case, edit, init_args, code, fragment", MODEL_CASES, ids=[c[0] for c in MODEL_CASES])
def test_model_loader_rejections(tmp_path, case, edit, init_args, code, fragment):
    """GAP XML checks of the model loader (IPModel_GAP.f95:618-944 reads the same
    stanzas), each raised before any device use, with its status and message."""
    L = _lib.load()
    xml = edit(_water_copy(tmp_path), tmp_path).encode()
    h = ctypes.c_void_p()
    rc = L.gapgpu_model_create(xml, len(xml), init_args.encode(), str(tmp_path).encode(), ctypes.byref(h))
    assert rc == getattr(_lib, code), (rc, L.gapgpu_last_error())
    assert fragment.encode() in L.gapgpu_last_error()
    assert not h.value


SOAP_BASE = "soap cutoff=4 cutoff_transition_width=1 n_max=4 l_max=4 atom_sigma=0.5 central_weight=1 " \
            "n_species=1 species_Z={14} n_Z=1 Z={14}"
# (case, descriptor string, dimensions written, expected status, message fragment)
SOAP_CASES = [
    ("valid", SOAP_BASE, 51, "ERR_CUDA", ""),
    ("n_max", SOAP_BASE.replace("n_max=4", "n_max=17"), 51, "ERR_UNSUPPORTED", "n_max outside"),
    ("l_max", SOAP_BASE.replace("l_max=4", "l_max=13"), 51, "ERR_UNSUPPORTED", "l_max outside"),
    ("n_species", SOAP_BASE.replace("n_species=1", "n_species=9"), 51, "ERR_UNSUPPORTED", "n_species outside"),
    ("diagonal_radial", SOAP_BASE + " diagonal_radial=T", 51, "ERR_UNSUPPORTED", "diagonal_radial"),
    ("average", SOAP_BASE + " average=T", 51, "ERR_UNSUPPORTED", "option average"),
    ("cutoff_dexp", SOAP_BASE + " cutoff_dexp=2", 51, "ERR_UNSUPPORTED", "cutoff_dexp"),
    ("species_Z short", SOAP_BASE.replace("n_species=1", "n_species=2"), 51, "ERR_XML", "species_Z shorter"),
    ("n_Z", SOAP_BASE.replace("n_Z=1", "n_Z=2"), 51, "ERR_XML", "inconsistent n_Z"),
    ("cutoff", SOAP_BASE.replace("cutoff=4 ", "cutoff=0 "), 51, "ERR_XML", "cutoff missing or not positive"),
    ("dimensions", SOAP_BASE, 50, "ERR_XML", "soap dimension mismatch"),
]


@pytest.mark.parametrize("case, desc, D, code, fragment", SOAP_CASES, ids=[c[0] for c in SOAP_CASES])
def test_soap_descriptor_checks(tmp_path, case, desc, D, code, fragment):
    """The SOAP descriptor string is read with GAP's keys and defaults; options the
    GPU path does not implement are refused rather than ignored."""
    L = _lib.load()
    p = models.write_gap_xml(str(tmp_path / "s.xml"), [dict(desc_str=desc, cov="dot_product", delta=1.0, zeta=2.0,
                                                            X=np.ones((3, D)), alpha=np.ones(3), sc=np.ones(3))])
    xml = open(p, "rb").read()
    h = ctypes.c_void_p()
    rc = L.gapgpu_model_create(xml, len(xml), b"", str(tmp_path).encode(), ctypes.byref(h))
    if rc == 0 and code == "ERR_CUDA":  # a GPU is present: the valid model is created
        L.gapgpu_model_destroy(h)
        return
    assert rc == getattr(_lib, code), (rc, L.gapgpu_last_error())
    assert fragment.encode() in L.gapgpu_last_error()


def test_unmodified_water_model_parses(tmp_path):
    """The same files unmodified get past every check; without a GPU the upload then
    fails with GAPGPU_ERR_CUDA (with one, the model is created)."""
    L = _lib.load()
    xml = _water_copy(tmp_path).encode()
    h = ctypes.c_void_p()
    rc = L.gapgpu_model_create(xml, len(xml), b"", str(tmp_path).encode(), ctypes.byref(h))
    if rc == 0:
        L.gapgpu_model_destroy(h)
    else:
        assert rc == _lib.ERR_CUDA, L.gapgpu_last_error()


def test_no_gpu_means_loud_failure(tmp_path):
    """No CPU fallback: without a GPU, model creation fails with GAPGPU_ERR_CUDA."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    from quip_gb300.potential import Potential
    from quip_gb300._lib import GapGpuError
    with pytest.raises(GapGpuError) as ei:
        Potential(param_filename=os.path.join(ROOT, "tests", "golden", "gap_water", "GAP.xml"))
    assert ei.value.code == _lib.ERR_CUDA


def test_xml_writer_round_trip_through_oracle_reader(tmp_path):
    rng = np.random.default_rng(0)
    X = rng.normal(size=(7, 51))
    desc = models.soap_descriptor_string(3.0, 4, 4, species=(14,))
    p = models.write_gap_xml(str(tmp_path / "m.xml"),
                             [dict(desc_str=desc, cov="dot_product", delta=2.0, zeta=3.0, X=X, alpha=np.arange(7.0),
                                   sc=np.ones(7)),
                              dict(desc_str="distance_2b cutoff=4.0 Z1=14 Z2=14", cov="ard_se", delta=0.5,
                                   theta=np.array([1.5]), X=np.linspace(1, 4, 5)[:, None], alpha=np.ones(5),
                                   sc=np.ones(5))], e0={14: -1.25})
    d = oracle.read_gap_xml(p)
    assert d["e0"][14] == -1.25
    c0, c1 = d["coords"]
    np.testing.assert_array_equal(c0["X"], X)
    assert c0["zeta"] == 3.0 and c0["delta"] == 2.0 and c0["cov"] == 2
    assert c1["cov"] == 1 and c1["theta"][0] == 1.5
    assert models.soap_dim(4, 4, 1) == c0["D"] == 51


def test_structure_generators():
    at = models.si_diamond(2, rattle=0.0)
    assert len(at) == 64 and abs(at.volume() - 10.86 ** 3) < 1e-9
    prim = models.si_primitive()
    assert len(prim) == 2
    w = 1.0 / np.linalg.norm(np.linalg.inv(prim.lattice), axis=1)
    assert w.max() < 5.0  # cutoff larger than the cell
    b = models.random_binary(400, seed=1)
    assert abs(len(b) / b.volume() - 0.0961) < 2e-3
    off, j, sh, d, r = oracle.neighbours(b.positions, b.lattice, [1, 1, 1], 1.6)
    assert len(r) == 0  # minimum separation holds
    t = models.random_triclinic(30, rng=np.random.default_rng(2))
    ang = [np.degrees(np.arccos(t.lattice[:, a] @ t.lattice[:, c] / np.linalg.norm(t.lattice[:, a]) /
                                np.linalg.norm(t.lattice[:, c]))) for a, c in ((0, 1), (0, 2), (1, 2))]
    assert all(60 < x < 120 for x in ang)


def test_oracle_neighbour_semantics():
    """QUIP semantics: no minimum image, all images inside the cutoff, strict '<'."""
    prim = models.si_primitive()
    off, j, sh, d, r = oracle.neighbours(prim.positions, prim.lattice, [1, 1, 1], 5.0)
    # brute force over images
    cnt = 0
    for a in range(2):
        for b in range(2):
            for s in np.ndindex(9, 9, 9):
                s = np.array(s) - 4
                v = prim.positions[b] + prim.lattice @ s - prim.positions[a]
                if (a != b or s.any()) and np.linalg.norm(v) < 5.0:
                    cnt += 1
    assert cnt == len(r)
    assert np.all(r < 5.0)
    # self images are present
    assert np.any((j[off[0]:off[1]] == 0))


def _brute_force_pairs(pos, lat, pbc, rc):
    """Every (i, j, shift) with |pos_j + L shift - pos_i| < rc, shift 0 along
    non-periodic axes, the exact self at zero shift excluded: QUIP's pair set, enumerated
    over a shift range wide enough for the cutoff (perpendicular heights of the cell)."""
    vol = abs(np.linalg.det(lat))
    a, b, c = lat[:, 0], lat[:, 1], lat[:, 2]
    heights = [vol / np.linalg.norm(np.cross(b, c)), vol / np.linalg.norm(np.cross(c, a)),
               vol / np.linalg.norm(np.cross(a, b))]
    frac = np.linalg.solve(lat, pos.T).T
    spread = frac.max(0) - frac.min(0)      # atoms may sit several cells apart
    K = [int(np.ceil(rc / heights[k] + spread[k])) + 1 if pbc[k] else 0 for k in range(3)]
    shifts = np.array(np.meshgrid(*[np.arange(-k, k + 1) for k in K], indexing="ij")).reshape(3, -1).T
    out = set()
    for i in range(len(pos)):
        d = pos[None, :, :] - pos[i] + (shifts @ lat.T)[:, None, :]   # [shift, j, 3]
        s_idx, js = np.nonzero(np.linalg.norm(d, axis=2) < rc)
        for s, j in zip(s_idx, js):
            if j == i and not shifts[s].any():
                continue
            out.add((i, int(j)) + tuple(int(x) for x in shifts[s]))
    return out


@pytest.mark.parametrize("seed", range(40))
def test_oracle_neighbours_against_brute_force(seed):
    """Random triclinic cells (lengths 2.5-8 A, angles 60-120 deg), random periodic flags,
    atoms up to two cells outside the cell, cutoffs below and above the cell widths: the
    oracle's list (Connection.f95 restated) is exactly the brute-force pair set."""
    rng = np.random.default_rng(1000 + seed)
    L = rng.uniform(2.5, 8.0, 3)
    al, be, ga = np.radians(rng.uniform(60, 120, 3))
    a = np.array([L[0], 0, 0])
    b = L[1] * np.array([np.cos(ga), np.sin(ga), 0])
    cx = np.cos(be)
    cy = (np.cos(al) - np.cos(be) * np.cos(ga)) / np.sin(ga)
    c = L[2] * np.array([cx, cy, np.sqrt(max(1e-3, 1 - cx * cx - cy * cy))])
    lat = np.stack([a, b, c], axis=1)
    n = int(rng.integers(1, 9))
    frac = rng.uniform(-2.0, 3.0, (n, 3))
    pbc = rng.integers(0, 2, 3)
    if seed % 4 == 0:
        pbc[:] = 1
    pos = frac @ lat.T
    rc = float(rng.uniform(1.5, 7.0))
    off, j, sh, d, r = oracle.neighbours(pos, lat, pbc, rc)
    got = {(i, int(j[p])) + tuple(int(x) for x in sh[p]) for i in range(n) for p in range(off[i], off[i + 1])}
    assert len(got) == len(j)                   # no pair listed twice
    assert got == _brute_force_pairs(pos, lat, pbc, rc)


def test_descriptor_string_parsing():
    d = models.soap_descriptor_string(5.0, 10, 8, species=(14, 6))
    a = models.parse_descriptor(d)
    assert a["species_Z"] == "14 6" and a["n_species"] == "2" and a["soap"] is True
    assert models.descriptor_dim(d) == 1891
    assert models.descriptor_dim(models.soap_descriptor_string(5.0, 8, 6)) == 253
    assert models.descriptor_dim("distance_2b cutoff=4 Z1=1 Z2=8") == 1


def test_extxyz_write_read_round_trip(tmp_path, golden):
    from quip_gb300.atoms import read_xyz, write_xyz
    frames = read_xyz(os.path.join(golden, "Si.np1.xyz"))[:4]
    t = models.random_triclinic(20, rng=np.random.default_rng(3))
    t.arrays["force"] = np.random.default_rng(4).normal(size=(20, 3))
    t.info["energy"] = -12.5
    p = str(tmp_path / "out.xyz")
    write_xyz(p, frames + [t])
    back = read_xyz(p)
    assert len(back) == 5
    for a, b in zip(frames + [t], back):
        np.testing.assert_array_equal(a.numbers, b.numbers)
        np.testing.assert_array_equal(a.positions, b.positions)
        np.testing.assert_array_equal(a.lattice, b.lattice)
        np.testing.assert_array_equal(a.pbc, b.pbc)
    np.testing.assert_array_equal(back[-1].arrays["force"], t.arrays["force"])
    assert back[-1].info["energy"] == -12.5

