"""Atoms container and extended-XYZ reader for the GAP path.

Mirrors the parts of QUIP's Atoms type that the GAP path reads
(src/libAtoms/Atoms_types.f95:224-347): N, Z(N), pos(3,N), lattice(3,3) whose
COLUMNS are the cell vectors, and is_periodic(3).  Positions are held as an
(N, 3) C-ordered array (row i = atom i), which is the same memory as Fortran
pos(3,N).  The extended-XYZ reader follows the header conventions that the
reference's C reader accepts (src/libAtoms/xyz.c): Lattice="..." gives the three
cell vectors in order, Properties=name:type:count:... describes the columns.
"""
import re

import numpy as np

SYMBOLS = ("X H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
           "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb Lu "
           "Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U Np Pu Am Cm Bk Cf Es Fm Md No Lr Rf Db Sg "
           "Bh Hs Mt Ds Rg Cn Nh Fl Mc Lv Ts Og").split()
Z_OF = {s: z for z, s in enumerate(SYMBOLS)}


class Atoms:
    """numbers (N,), positions (N,3), lattice (3,3) with columns = cell vectors, pbc (3,)."""

    def __init__(self, numbers, positions, lattice=None, cell=None, pbc=True, info=None, arrays=None):
        self.numbers = np.ascontiguousarray(numbers, dtype=np.int32)
        self.positions = np.ascontiguousarray(positions, dtype=np.float64).reshape(-1, 3)
        if lattice is None and cell is None:
            raise ValueError("Atoms needs a lattice (columns = cell vectors) or a cell (rows = cell vectors)")
        if lattice is None:
            lattice = np.asarray(cell, dtype=np.float64).T
        self.lattice = np.array(lattice, dtype=np.float64).reshape(3, 3)
        p = np.broadcast_to(np.asarray(pbc, dtype=bool), (3,))
        self.pbc = np.array(p, dtype=bool)
        self.info = dict(info or {})
        self.arrays = dict(arrays or {})
        if len(self.numbers) != len(self.positions):
            raise ValueError("numbers and positions differ in length")

    def __len__(self):
        return len(self.numbers)

    @property
    def cell(self):
        """Rows = cell vectors (ASE convention)."""
        return self.lattice.T.copy()

    def volume(self):
        return abs(np.linalg.det(self.lattice))

    def copy(self):
        return Atoms(self.numbers.copy(), self.positions.copy(), lattice=self.lattice.copy(), pbc=self.pbc.copy(),
                     info=dict(self.info), arrays={k: v.copy() for k, v in self.arrays.items()})


_TYPES = {"R": float, "I": int, "S": str, "L": lambda v: v.upper().startswith("T")}


def _parse_header(hdr):
    kv = {}
    for m in re.finditer(r'(\w+)=("([^"]*)"|\S+)', hdr):
        kv[m.group(1)] = m.group(3) if m.group(3) is not None else m.group(2)
    return kv


def read_xyz(path, index=None):
    """Read every frame (or frame `index`) of an extended-XYZ file."""
    frames = []
    with open(path) as f:
        lines = f.read().splitlines()
    i = 0
    while i < len(lines):
        if not lines[i].strip():
            i += 1
            continue
        n = int(lines[i].split()[0])
        kv = _parse_header(lines[i + 1])
        props = kv.get("Properties", "species:S:1:pos:R:3").split(":")
        cols = []
        c = 0
        for k in range(0, len(props), 3):
            name, typ, cnt = props[k], props[k + 1], int(props[k + 2])
            cols.append((name, typ, c, cnt))
            c += cnt
        data = [l.split() for l in lines[i + 2:i + 2 + n]]
        arrays = {}
        for name, typ, c0, cnt in cols:
            conv = _TYPES[typ]
            vals = [[conv(row[c0 + k]) for k in range(cnt)] for row in data]
            arr = np.array(vals, dtype=object if typ == "S" else None)
            arrays[name] = arr[:, 0] if cnt == 1 else arr
        if "Z" in arrays:
            numbers = np.asarray(arrays["Z"], dtype=np.int32)
        else:
            numbers = np.array([Z_OF[str(s)] for s in arrays["species"]], dtype=np.int32)
        pos = np.asarray(arrays["pos"], dtype=np.float64)
        info = {}
        for k, v in kv.items():
            if k in ("Lattice", "Properties", "pbc"):
                continue
            try:
                info[k] = float(v)
            except ValueError:
                info[k] = v
        if "Lattice" in kv:
            lat = np.array([float(x) for x in kv["Lattice"].split()]).reshape(3, 3).T
            pbc = [s.upper().startswith("T") for s in kv.get("pbc", "T T T").split()]
        else:
            lat = np.eye(3) * (np.ptp(pos, axis=0).max() + 10.0)
            pbc = [False, False, False]
        frames.append(Atoms(numbers, pos, lattice=lat, pbc=pbc, info=info, arrays=arrays))
        i += 2 + n
    if index is not None:
        return frames[index]
    return frames


def _fmt_value(v):
    if isinstance(v, (bool, np.bool_)):
        return "T" if v else "F"
    if isinstance(v, (int, np.integer)):
        return "%d" % v
    if isinstance(v, (float, np.floating)):
        return "%.17g" % v
    v = str(v)
    return '"%s"' % v if (" " in v or "=" in v) else v


def write_xyz(path, frames, properties=("force",), mode="w"):
    """Write frames as extended XYZ in the header conventions read_xyz (and the
    reference's reader, src/libAtoms/xyz.c) accept: Lattice="..." (cell vectors in
    order), Properties=species:S:1:pos:R:3[:name:R:k...], pbc="T T T", info entries as
    key=value.  Per-atom arrays named in `properties` are written when present (N or
    N x k floats).  Positions and floats keep 17 significant digits, so a write/read
    round trip is exact."""
    if isinstance(frames, Atoms):
        frames = [frames]
    with open(path, mode) as f:
        for at in frames:
            extra = []
            for name in properties:
                if name in at.arrays:
                    a = np.asarray(at.arrays[name], dtype=np.float64)
                    extra.append((name, a.reshape(len(at), -1)))
            props = "species:S:1:pos:R:3" + "".join(":%s:R:%d" % (nm, a.shape[1]) for nm, a in extra)
            hdr = ['Lattice="%s"' % " ".join("%.17g" % x for x in at.lattice.T.ravel()),
                   "Properties=%s" % props, 'pbc="%s"' % " ".join("T" if p else "F" for p in at.pbc)]
            hdr += ["%s=%s" % (k, _fmt_value(v)) for k, v in at.info.items()]
            f.write("%d\n%s\n" % (len(at), " ".join(hdr)))
            for i in range(len(at)):
                cols = [SYMBOLS[int(at.numbers[i])]] + ["%.17g" % x for x in at.positions[i]]
                for _, a in extra:
                    cols += ["%.17g" % x for x in a[i]]
                f.write(" ".join(cols) + "\n")

