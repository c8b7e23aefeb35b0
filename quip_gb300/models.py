"""Seeded synthetic structures and random GAP models, written in gap_fit's XML format.

The reference publishes no benchmark dataset for the GAP path; these generators are
the stand-in workloads with the shapes, sizes and value distributions of the
benchmark configurations:
  * Si diamond supercells (a = 5.43 A) rattled by N(0, sigma) -- 64 and 4096 atoms;
  * the 2-atom primitive Si cell (cutoff larger than the cell);
  * a random binary Si/C cell at 3.2 g/cm^3 with a minimum separation;
  * batches of random triclinic Si/C cells with log-uniform atom counts.
Random models follow the gap_fit file layout (IPModel_GAP.f95:618-944,
quippy/quippy/gap_tools.py:17-75): GAP_params/GAP_data/e0, gpSparse/gpCoordinates with
descriptor string, sparseX attributes and an external sparseX file of M*D values.
"""
import os

import numpy as np

from .atoms import Atoms

GAP_VERSION = 1527075646
MASS = {1: 1.008, 6: 12.011, 8: 15.999, 14: 28.0855}


# ------------------------------------------------------------------ structures
def si_diamond(n_rep=2, a=5.43, rattle=0.05, seed=0):
    """Conventional 8-atom diamond cell replicated n_rep^3 times, rattled by N(0, rattle)."""
    basis = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0],
                      [.25, .25, .25], [.25, .75, .75], [.75, .25, .75], [.75, .75, .25]])
    g = np.stack(np.meshgrid(*[np.arange(n_rep)] * 3, indexing="ij"), -1).reshape(-1, 3)
    frac = (g[:, None, :] + basis[None, :, :]).reshape(-1, 3) / n_rep
    L = a * n_rep
    pos = frac * L
    rng = np.random.default_rng(seed)
    pos = pos + rng.normal(0.0, rattle, pos.shape)
    return Atoms(np.full(len(pos), 14), pos, lattice=np.eye(3) * L, pbc=True)


def si_primitive(a=5.43, rattle=0.0, seed=0):
    """2-atom fcc primitive Si cell: perpendicular width ~3.13 A, below a 5 A cutoff."""
    lat = 0.5 * a * np.array([[0, 1, 1], [1, 0, 1], [1, 1, 0]], dtype=float).T  # columns
    pos = np.array([lat @ np.array([0.0, 0.0, 0.0]), lat @ np.array([0.25, 0.25, 0.25])])
    rng = np.random.default_rng(seed)
    pos = pos + rng.normal(0.0, rattle, pos.shape)
    return Atoms([14, 14], pos, lattice=lat, pbc=True)


def _place_uniform(n, lat, min_sep, rng, batch=256, max_stall=200):
    """Random sequential addition with a minimum separation (periodic, any lattice),
    in batches: a batch of uniform candidates is tested against every accepted atom in
    the 27 neighbouring cells of a grid at least min_sep wide, then accepted in order
    unless it clashes with an earlier candidate of the same batch.  Distances use the
    nearest image in fractional coordinates, and all 27 images when the cell is less
    than three grid cells wide."""
    g = np.linalg.inv(lat)
    widths = 1.0 / np.linalg.norm(g, axis=1)  # perpendicular widths
    nb = np.maximum(1, (widths / min_sep).astype(int))
    small = nb.min() < 3
    shifts = np.array([[i, j, k] for i in (-1, 0, 1) for j in (-1, 0, 1) for k in (-1, 0, 1)])
    ncell = int(np.prod(nb))
    cap = 8
    cell_atoms = np.full((ncell, cap), -1, dtype=np.int64)
    cell_cnt = np.zeros(ncell, dtype=np.int64)
    frac = np.zeros((n, 3))
    ms2 = min_sep * min_sep
    m, stall = 0, 0

    def r2_of(d):  # squared Cartesian length of fractional differences (..., 3), nearest image
        d = d - np.round(d)
        if not small:
            c = d @ lat.T
            return np.einsum("...i,...i->...", c, c)
        c = (d[..., None, :] + shifts) @ lat.T
        return np.einsum("...i,...i->...", c, c).min(axis=-1)

    while m < n:
        k = min(batch, 2 * (n - m) + 8)
        cand = rng.random((k, 3))
        ci = (cand * nb).astype(np.int64) % nb
        nc = (ci[:, None, :] + shifts[None]) % nb
        lin = nc[..., 0] + nb[0] * (nc[..., 1] + nb[1] * nc[..., 2])
        idx = cell_atoms[lin].reshape(k, -1)
        valid = idx >= 0
        r2 = np.where(valid, r2_of(frac[np.where(valid, idx, 0)] - cand[:, None, :]), np.inf)
        sel = np.nonzero(r2.min(axis=1) >= ms2)[0]
        took = 0
        if len(sel):
            C = cand[sel]
            clash = r2_of(C[:, None, :] - C[None, :, :]) < ms2
            np.fill_diagonal(clash, False)
            taken = np.zeros(len(sel), dtype=bool)
            for i in range(len(sel)):
                if m + took >= n:
                    break
                if not (clash[i] & taken).any():
                    taken[i] = True
                    took += 1
            for i in np.nonzero(taken)[0]:
                c = int(lin[sel[i], 13])  # the candidate's own cell (zero shift)
                if cell_cnt[c] == cap:
                    cap *= 2
                    grown = np.full((ncell, cap), -1, dtype=np.int64)
                    grown[:, :cap // 2] = cell_atoms
                    cell_atoms = grown
                cell_atoms[c, cell_cnt[c]] = m
                cell_cnt[c] += 1
                frac[m] = C[i]
                m += 1
        stall = 0 if took else stall + 1
        if stall > max_stall:
            raise RuntimeError("could not place atom %d with min separation %.2f" % (m, min_sep))
    return frac @ lat.T


def random_binary(n=32768, density_gcc=3.2, min_sep=1.6, species=(14, 6), seed=0):
    """Cubic random Si/C cell, 50/50, uniform positions with a minimum separation."""
    rng = np.random.default_rng(seed)
    Z = np.array([species[k % 2] for k in range(n)])
    rng.shuffle(Z)
    mass = np.mean([MASS[z] for z in species])
    nd = density_gcc / mass * 0.602214076  # atoms / A^3
    L = (n / nd) ** (1.0 / 3.0)
    lat = np.eye(3) * L
    pos = _place_uniform(n, lat, min_sep, rng)
    return Atoms(Z, pos, lattice=lat, pbc=True)


def random_triclinic(n, species=(14, 6), min_sep=1.8, max_density=0.08, rng=None):
    """Random triclinic cell (lengths 4-30 A, angles 70-110 deg) holding n atoms."""
    rng = rng or np.random.default_rng(0)
    for _ in range(1000):
        lens = rng.uniform(4.0, 30.0, 3)
        al, be, ga = np.radians(rng.uniform(70.0, 110.0, 3))
        a = np.array([lens[0], 0.0, 0.0])
        b = lens[1] * np.array([np.cos(ga), np.sin(ga), 0.0])
        cx = np.cos(be)
        cy = (np.cos(al) - np.cos(be) * np.cos(ga)) / np.sin(ga)
        cz2 = 1.0 - cx * cx - cy * cy
        if cz2 <= 0.05:
            continue
        c = lens[2] * np.array([cx, cy, np.sqrt(cz2)])
        lat = np.stack([a, b, c], axis=1)
        vol = abs(np.linalg.det(lat))
        if n / vol <= max_density:
            break
        # scale the cell up to the density bound
        s = (n / (vol * max_density)) ** (1.0 / 3.0)
        lat = lat * s
        if np.all(np.linalg.norm(lat, axis=0) <= 30.0 * 2.5):
            break
    Z = rng.choice(np.array(species), n)
    for _ in range(20):  # random sequential addition can jam: retry in a 5% larger cell
        try:
            pos = _place_uniform(n, lat, min_sep, rng)
            break
        except RuntimeError:
            lat = lat * 1.05
    else:
        raise RuntimeError("could not place %d atoms with minimum separation %.2f" % (n, min_sep))
    return Atoms(Z, pos, lattice=lat, pbc=True)


def _triclinic_item(args):
    k, n, seed, kw = args
    return random_triclinic(int(n), rng=np.random.default_rng([seed, k]), **kw)


def triclinic_batch(count=1024, n_min=8, n_max=2048, seed=0, workers=1, **kw):
    """`count` random triclinic Si/C cells with atom counts log-uniform in [n_min, n_max].
    Structure k is drawn from its own seed (seed, k), so the batch is the same whatever
    the number of worker processes (spawned, so that no GPU context is forked)."""
    rng = np.random.default_rng(seed)
    ns = np.exp(rng.uniform(np.log(n_min), np.log(n_max), count)).astype(int)
    items = [(k, int(n), seed, kw) for k, n in enumerate(ns)]
    if workers <= 1:
        return [_triclinic_item(it) for it in items]
    import concurrent.futures as cf
    import multiprocessing as mp
    with cf.ProcessPoolExecutor(max_workers=workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_triclinic_item, items, chunksize=8))


# ------------------------------------------------------------------ GAP XML
def soap_descriptor_string(cutoff, n_max, l_max, atom_sigma=0.5, width=1.0, species=(14,), centres=None,
                           central_weight=1.0):
    centres = species if centres is None else centres
    return ("soap cutoff=%g cutoff_transition_width=%g n_max=%d l_max=%d atom_sigma=%g central_weight=%g "
            "n_species=%d species_Z={%s} n_Z=%d Z={%s}" % (cutoff, width, n_max, l_max, atom_sigma, central_weight,
                                                            len(species), " ".join(map(str, species)), len(centres),
                                                            " ".join(map(str, centres))))


def parse_descriptor(desc):
    """key=value pairs of a descriptor string; values may be {..} lists or quoted."""
    import re
    out = {}
    for k, v, bare in re.findall(r'(\S+?)=(\{[^}]*\}|"[^"]*"|\S+)|(\S+)', desc):
        if bare:
            out[bare] = True
        else:
            out[k] = v[1:-1].strip() if v[:1] in "{\"" else v
    return out


def descriptor_dim(desc):
    a = parse_descriptor(desc)
    if "soap" in a:
        ns = int(a.get("n_species", 1))
        return soap_dim(int(a.get("n_max", 4)), int(a.get("l_max", 4)), ns)
    if "distance_2b" in a:
        return 1
    raise ValueError("unknown descriptor %r" % desc)


def soap_dim(n_max, l_max, n_species):
    N = n_max * n_species
    return (l_max + 1) * N * (N + 1) // 2 + 1


def write_gap_xml(path, coords, e0=None, label="GB300_GAP"):
    """coords: list of dicts with desc_str, cov ('ard_se'|'dot_product'), delta, zeta,
    theta (ard_se), X (M,D), alpha (M,), sc (M,) -- written as gap_fit does."""
    e0 = e0 or {}
    base = os.path.dirname(os.path.abspath(path))
    fn = os.path.basename(path)
    out = ['<%s>' % label,
           '<Potential label="%s" init_args="IP GAP label=%s"/>' % (label, label),
           '<GAP_params label="%s" gap_version="%d">' % (label, GAP_VERSION),
           '  <GAP_data do_core="F">']
    for z in range(1, 117):
        out.append('    <e0 Z="%d" value="%.17e"/>' % (z, e0.get(z, 0.0)))
    out.append('  </GAP_data>')
    out.append('  <gpSparse label="%s" n_coordinate="%d">' % (label, len(coords)))
    for k, c in enumerate(coords):
        X = np.asarray(c["X"], dtype=np.float64).reshape(len(c["alpha"]), -1)
        M, D = X.shape
        sname = "%s.sparseX.%s%d" % (fn, label, k + 1)
        X.reshape(-1).tofile(os.path.join(base, sname), sep="\n", format="%.20e")
        cov = {"ard_se": 1, "dot_product": 2}[c["cov"]]
        zeta = ' zeta="%.17e"' % c["zeta"] if cov == 2 else ""
        out.append('    <gpCoordinates label="%s%d" dimensions="%d" signal_variance="%.17e" signal_mean="0.0" '
                   'sparsified="T" n_permutations="1" covariance_type="%d"%s n_sparseX="%d" sparseX_filename="%s">'
                   % (label, k + 1, D, c["delta"], cov, zeta, M, sname))
        if cov == 1:
            out.append('      <theta>%s</theta>' % " ".join("%.17e" % t for t in np.atleast_1d(c["theta"])))
        out.append('      <descriptor>%s</descriptor>' % c["desc_str"])
        out.append('      <permutation i="1">%s</permutation>' % " ".join(str(i + 1) for i in range(D)))
        sc = np.ones(M) if c.get("sc") is None else c["sc"]
        for s in range(M):
            out.append('      <sparseX i="%d" alpha="%.17e" sparseCutoff="%.17e"/>' % (s + 1, c["alpha"][s], sc[s]))
        out.append('    </gpCoordinates>')
    out += ['  </gpSparse>', '</GAP_params>', '</%s>' % label]
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    return path


def random_soap_gap(path, descriptor_fn, structures, n_max=8, l_max=6, cutoff=5.0, width=1.0, atom_sigma=0.5,
                    species=(14,), M=500, zeta=4.0, delta=1.0, alpha_sigma=1e-3, with_2b=True, M2=20, theta2=1.0,
                    seed=0, e0=None):
    """Random GAP model: sparse points are normalised SOAP vectors of `structures`
    (computed by descriptor_fn(desc_str, atoms) -> (n_centres, D)), alpha ~ N(0, alpha_sigma);
    plus distance_2b with M2 uniform sparse distances and ard_se theta2."""
    rng = np.random.default_rng(seed)
    desc = soap_descriptor_string(cutoff, n_max, l_max, atom_sigma, width, species)
    Q = np.concatenate([descriptor_fn(desc, at) for at in structures], axis=0)
    if len(Q) < M:
        raise ValueError("need at least %d descriptor vectors, got %d" % (M, len(Q)))
    X = Q[rng.choice(len(Q), M, replace=False)]
    coords = [dict(desc_str=desc, cov="dot_product", delta=delta, zeta=zeta, X=X, alpha=rng.normal(0, alpha_sigma, M),
                   sc=np.ones(M))]
    if with_2b:
        for a, zi in enumerate(species):
            for zj in species[a:]:
                x = np.linspace(1.5, cutoff, M2)
                coords.append(dict(desc_str="distance_2b cutoff=%g cutoff_transition_width=1.0 Z1=%d Z2=%d"
                                   % (cutoff, zi, zj), cov="ard_se", delta=1.0, theta=np.array([theta2]),
                                   X=x[:, None], alpha=rng.normal(0, alpha_sigma, M2), sc=np.ones(M2)))
    e0 = e0 if e0 is not None else {z: -0.1 * (k + 1) for k, z in enumerate(species)}
    return write_gap_xml(path, coords, e0=e0)


def bootstrap_descriptor_fn(precision="fp64"):
    """descriptor_fn that computes SOAP vectors on the GPU through a one-point model."""
    import tempfile
    from .potential import Potential

    cache = {}

    def fn(desc, at):
        if desc not in cache:
            d = tempfile.mkdtemp(prefix="gapboot")
            D = descriptor_dim(desc)
            p = write_gap_xml(os.path.join(d, "boot.xml"),
                              [dict(desc_str=desc, cov="dot_product", delta=1.0, zeta=1.0,
                                    X=np.eye(1, D), alpha=np.zeros(1), sc=np.ones(1))])
            cache[desc] = Potential(param_filename=p, precision=precision)
        return cache[desc].descriptors(at, 0)

    return fn
